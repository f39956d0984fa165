// Request server: forward, adjoint and operator-norm requests on resident
// coverages, admitted by an HBM budget and run concurrently.
//
// A coverage (an Operator: sorted uv, weights, kernel fit, task lists) is
// built once and stays on the device.  A request brings only its own data; on
// admission it receives its own workspace (padded and FFT grids, task
// windows, slot buffer, I/O vectors) from a stream-ordered device memory pool
// and one of `slots` CUDA streams, so requests that arrive while others run
// are admitted as streams and memory free up, and their kernels overlap on
// the GPU.  Nothing a request reads or writes is shared with another
// request, so its result does not depend on what else is in flight.
#pragma once
#include <cuda_runtime_api.h>
#include <cufft.h>

#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "operator.h"

namespace pg {

enum RequestKind : int {
  kReqForward = 1,         // vis_out = Phi x_in
  kReqAdjoint = 2,         // x_out = Phi^H vis_in  (dirty image)
  kReqForwardAdjoint = 3,  // vis_out = Phi x_in, x_out = Phi^H vis_out
  kReqNorm = 4,            // ||Phi'|| by `iters` power-method rounds
};

struct ServerConfig {
  int device = 0;
  int slots = 8;                  // requests in flight at most (one stream each)
  int64_t hbm_budget = 8LL << 30; // device bytes of the requests in flight
  // Slots norm requests (many rounds each) may hold at once; 0: a quarter of
  // the slots, at least one.  They run on low-priority streams, the other
  // requests on high-priority ones, so the block scheduler serves short
  // requests first when both wait.
  int norm_slots = 0;
};

// Host buffers are complex<double> (interleaved), as the host entry points.
struct Request {
  int coverage = 0;
  int kind = kReqForwardAdjoint;
  const double *x_in = nullptr;   // imsizey * imsizex (forward kinds)
  const double *vis_in = nullptr; // M (adjoint)
  double *vis_out = nullptr;      // M (forward kinds)
  double *x_out = nullptr;        // imsizey * imsizex (adjoint kinds)
  int iters = 50;                 // norm
  double tol = 1e-4;              // norm: the single-operator stopping rule
};

struct RequestResult {
  int status = kOk;
  double norm = 0;
  int iterations = 0;
  double queue_ms = 0, run_ms = 0, latency_ms = 0;  // submit->admit, admit->done, submit->done
  int64_t device_bytes = 0;  // held while in flight
};

struct ServerStats {
  int64_t submitted = 0, completed = 0, rejected = 0, failed = 0;
  int64_t inflight_peak = 0, bytes_peak = 0, bytes_budget = 0;
  double latency_p50_ms = 0, latency_p99_ms = 0, latency_mean_ms = 0;
  double visibility_passes = 0;  // sum over completed requests of M x (G and G^H passes)
};

class Server {
 public:
  explicit Server(const ServerConfig &cfg);
  ~Server();
  Server(const Server &) = delete;
  Server &operator=(const Server &) = delete;
  // Builds a resident coverage (with its norm when cfg.power_iters > 0);
  // returns its id.
  int add_coverage(const OperatorConfig &cfg);
  // Device bytes a request would hold while in flight.
  int64_t request_bytes(const Request &rq) const;
  // Queues the request (its input is copied at once, so the caller's input
  // buffer may be reused on return) and returns its ticket.  A request that
  // could never fit the budget completes at once with kRejected.
  int64_t submit(const Request &rq);
  // Waits up to timeout_s (< 0: forever) for the request; on completion
  // copies its outputs into the buffers named at submit, fills `out`, forgets
  // the ticket and returns true.
  bool wait(int64_t ticket, double timeout_s, RequestResult *out);
  ServerStats stats() const;

 private:
  struct Job;
  struct Slot;
  struct Coverage;
  void loop();
  void reserve(Job &job, Slot &slot);
  void work(Slot &slot);
  bool enqueue(Job &job, cufftHandle fft, cufftHandle fft_cols);
  void finish(Job &job);
  static void CUDART_CB on_done(void *job);
  void *pinned(size_t bytes);
  void unpin(void *p, size_t bytes);

  ServerConfig cfg_;
  const Coverage &coverage(int id) const;
  std::vector<std::unique_ptr<Coverage>> coverages_;  // appended under cov_mu_
  mutable std::mutex cov_mu_;
  std::vector<std::unique_ptr<Slot>> slots_;
  cudaMemPool_t pool_ = nullptr;
  std::map<int64_t, std::shared_ptr<Job>> jobs_;
  std::deque<std::shared_ptr<Job>> pending_;
  std::deque<Job *> completed_;  // device work done, not yet retired
  int64_t next_ticket_ = 1, bytes_in_use_ = 0, inflight_ = 0;
  ServerStats stats_;
  std::vector<double> latencies_;
  std::multimap<size_t, void *> pinned_free_;
  mutable std::mutex mu_;
  int norm_slots_ = 1;  // slots that take norm requests (the first ones)
  std::condition_variable cv_;       // scheduler wake-ups
  std::condition_variable done_cv_;  // request completions
  bool stop_ = false, dirty_ = false, workers_stop_ = false;
  std::thread thread_;
};

}  // namespace pg
