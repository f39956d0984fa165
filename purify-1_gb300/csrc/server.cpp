#include "server.h"

#include <cufft.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <string>

#include "device_kernels.h"
#include "device_util.h"
#include "fft_kernels.h"

namespace pg {
namespace {

using Clock = std::chrono::steady_clock;
double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}
size_t up256(size_t b) { return (b + 255) / 256 * 256; }

// A non-head request may overtake a head that does not fit the budget at
// most this many times before admission waits for the head.
constexpr int kMaxOvertakes = 16;
// Power-method rounds of a norm request enqueued at a time (see enqueue).
constexpr int kNormChunk = 4;
// Pinned staging buffers of each size class a coverage uses, allocated when
// the coverage is added: pinning host memory takes milliseconds, too long for
// the submit path of a request.
constexpr int kPinnedWarm = 2;
size_t pinned_class(size_t bytes) {
  size_t cls = 4096;
  while (cls < bytes) cls <<= 1;
  return cls;
}

}  // namespace

struct Server::Coverage {
  std::unique_ptr<Operator> op;
  OperatorInfo info;
  WorkspaceSizes ws;
  int64_t M = 0, N = 0;
  bool fp64 = false;
};

struct Server::Slot {
  cudaStream_t stream = nullptr;
  std::map<int64_t, cufftHandle> plans;  // key: fp64 | Nu << 1 | Nv << 32
  std::map<int64_t, cufftHandle> col_plans;  // FP32 column transforms, same key
  bool busy = false;
  bool long_slot = false;  // serves norm requests (lowest stream priority)
  // The slot's enqueue thread: the scheduler hands it an admitted job, and
  // it enqueues the job's copies and launches on the slot's stream, so a
  // long request's launches do not hold up admission of the others.
  Job *job = nullptr;
  std::condition_variable cv;
  std::thread worker;
  cudaEvent_t chunk_ev[2] = {nullptr, nullptr};  // the last two norm pieces enqueued
};

struct Server::Job {
  Server *server = nullptr;
  int64_t ticket = 0;
  Request rq;
  int status = kOk;
  bool done = false;
  int overtaken = 0;
  Clock::time_point t_submit, t_admit, t_done;
  void *host_in = nullptr, *host_out = nullptr;
  size_t in_bytes = 0, out_bytes = 0;
  void *dev = nullptr;
  int64_t bytes = 0;
  Slot *slot = nullptr;
  double norm = 0;
  int iterations = 0;
};

// Host copies between the caller's vectors and pinned staging.  Large ones
// are split over host threads: a single thread's memcpy is well below the
// host memory bandwidth, and the submitting thread pays for it.
static void copy_bytes(void *dst, const void *src, size_t bytes) {
  constexpr size_t kParallelBytes = size_t(4) << 20;
  if (bytes < kParallelBytes) {
    std::memcpy(dst, src, bytes);
    return;
  }
  const int64_t pieces = int64_t((bytes + (size_t(1) << 20) - 1) >> 20);
#pragma omp parallel for schedule(static) num_threads(8)
  for (int64_t k = 0; k < pieces; ++k) {
    const size_t off = size_t(k) << 20;
    std::memcpy(static_cast<char *>(dst) + off, static_cast<const char *>(src) + off,
                std::min(size_t(1) << 20, bytes - off));
  }
}

static int64_t plan_key(bool fp64, int Nu, int Nv) {
  return int64_t(fp64) | (int64_t(Nu) << 1) | (int64_t(Nv) << 32);
}

Server::Server(const ServerConfig &cfg) : cfg_(cfg) {
  if (cfg.slots < 1 || cfg.slots > 64) throw Error(kInvalidArgument, "slots must be in [1, 64]");
  if (cfg.hbm_budget <= 0) throw Error(kInvalidArgument, "the HBM budget must be positive");
  DeviceGuard guard(cfg.device);
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = cfg.device;
  cuda_check(cudaMemPoolCreate(&pool_, &props), "cudaMemPoolCreate");
  // Keep freed request memory in the pool (no return to the driver between
  // requests); the budget bounds what is in use.
  uint64_t keep = uint64_t(cfg.hbm_budget);
  cuda_check(cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &keep),
             "cudaMemPoolSetAttribute");
  if (cfg.norm_slots < 0 || cfg.norm_slots > cfg.slots)
    throw Error(kInvalidArgument, "norm_slots must be in [0, slots]");
  norm_slots_ = cfg.norm_slots > 0 ? cfg.norm_slots : std::max(1, cfg.slots / 4);
  // The first norm_slots_ slots are the long-request (norm) slots, on the
  // lowest stream priority; the others on the highest.
  int lo = 0, hi = 0;
  cuda_check(cudaDeviceGetStreamPriorityRange(&lo, &hi), "cudaDeviceGetStreamPriorityRange");
  for (int k = 0; k < cfg.slots; ++k) {
    std::unique_ptr<Slot> s(new Slot);
    s->long_slot = k < norm_slots_;
    cuda_check(cudaStreamCreateWithPriority(&s->stream, cudaStreamNonBlocking,
                                            s->long_slot ? lo : hi),
               "cudaStreamCreateWithPriority");
    for (cudaEvent_t &e : s->chunk_ev)
      cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
    slots_.push_back(std::move(s));
  }
  stats_.bytes_budget = cfg.hbm_budget;
  for (auto &s : slots_) {
    Slot *sp = s.get();
    sp->worker = std::thread([this, sp] { work(*sp); });
  }
  thread_ = std::thread([this] { loop(); });
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
    dirty_ = true;
  }
  cv_.notify_all();
  if (thread_.joinable()) thread_.join();
  // every admitted job has been enqueued and retired by now
  {
    std::lock_guard<std::mutex> lk(mu_);
    workers_stop_ = true;
  }
  for (auto &s : slots_) s->cv.notify_all();
  for (auto &s : slots_)
    if (s->worker.joinable()) s->worker.join();
  DeviceGuard guard(cfg_.device);
  for (auto &s : slots_) {
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (auto &kv : s->plans) cufftDestroy(kv.second);
    for (auto &kv : s->col_plans) cufftDestroy(kv.second);
    for (cudaEvent_t e : s->chunk_ev)
      if (e) cudaEventDestroy(e);
    if (s->stream) cudaStreamDestroy(s->stream);
  }
  if (pool_) cudaMemPoolDestroy(pool_);
  for (auto &kv : jobs_) {
    Job &j = *kv.second;
    if (j.host_in) unpin(j.host_in, j.in_bytes);
    if (j.host_out) unpin(j.host_out, j.out_bytes);
  }
  for (auto &kv : pinned_free_) cudaFreeHost(kv.second);
}

int Server::add_coverage(const OperatorConfig &cfg_in) {
  OperatorConfig cfg = cfg_in;
  cfg.device = cfg_.device;
  std::unique_ptr<Coverage> c(new Coverage);
  c->op = Operator::create(cfg);
  c->info = c->op->info();
  c->ws = c->op->workspace_sizes();
  c->M = c->info.M;
  c->N = int64_t(c->info.imsizey) * c->info.imsizex;
  c->fp64 = c->info.fp64;
  // cuFFT plans of this grid size for every slot, made before any request
  // needs them (plan creation allocates).
  DeviceGuard guard(cfg_.device);
  const int64_t key = plan_key(c->fp64, int(c->info.ftsizeu), int(c->info.ftsizev));
  std::lock_guard<std::mutex> lk(mu_);
  for (auto &s : slots_) {
    if (!s->plans.count(key)) {
      cufftHandle h = 0;
      cufft_check(cufftPlan2d(&h, int(c->info.ftsizev), int(c->info.ftsizeu),
                              c->fp64 ? CUFFT_Z2Z : CUFFT_C2C),
                  "cufftPlan2d");
      const cufftResult r = cufftSetStream(h, s->stream);
      if (r != CUFFT_SUCCESS) {
        cufftDestroy(h);
        cufft_check(r, "cufftSetStream");
      }
      s->plans[key] = h;
    }
    // the cuFFT column transform of the fused FFT path, where the operator
    // does not run its own column pass (fft_kernels.h)
    if (c->op->needs_column_plan() && !s->col_plans.count(key))
      s->col_plans[key] =
          make_column_plan<float>(int(c->info.ftsizeu), int(c->info.ftsizev), s->stream, nullptr);
  }
  // staging of the request kinds' inputs and outputs: 16 N, 16 M, 16 (M + N)
  for (int64_t n : {16 * c->N, 16 * c->M, 16 * (c->M + c->N)}) {
    const size_t cls = pinned_class(size_t(std::max<int64_t>(n, 1)));
    while (int(pinned_free_.count(cls)) < kPinnedWarm) {
      void *p = nullptr;
      cuda_check(cudaHostAlloc(&p, cls, cudaHostAllocPortable), "cudaHostAlloc");
      pinned_free_.emplace(cls, p);
    }
  }
  std::lock_guard<std::mutex> ck(cov_mu_);
  coverages_.push_back(std::move(c));
  return int(coverages_.size()) - 1;
}

// Coverages are only ever appended and live as long as the server, so the
// reference stays valid after the lock is released.
const Server::Coverage &Server::coverage(int id) const {
  std::lock_guard<std::mutex> ck(cov_mu_);
  if (id < 0 || id >= int(coverages_.size())) throw Error(kInvalidArgument, "unknown coverage");
  return *coverages_[size_t(id)];
}

// Device layout of a request, 256-byte aligned pieces: complex<double> I/O
// vectors, their working-precision copies (FP32 only), the workspace, and the
// power-method vectors.
int64_t Server::request_bytes(const Request &rq) const {
  const Coverage &c = coverage(rq.coverage);
  const size_t cs = c.fp64 ? 16 : 8;
  size_t b = up256(size_t(c.ws.pad)) + up256(size_t(c.ws.work)) + up256(size_t(c.ws.tilebuf)) +
             up256(size_t(c.ws.slots));
  if (rq.kind == kReqNorm) {
    b += up256(cs * size_t(c.N)) + up256(sizeof(double) * std::max(rq.iters, 1)) +
         up256(sizeof(double) * kNormBlocks);
    return int64_t(b);
  }
  b += up256(16 * size_t(c.N)) + up256(16 * size_t(std::max<int64_t>(c.M, 1)));
  if (!c.fp64) b += up256(8 * size_t(c.N)) + up256(8 * size_t(std::max<int64_t>(c.M, 1)));
  return int64_t(b);
}

void *Server::pinned(size_t bytes) {
  const size_t cls = pinned_class(bytes);
  {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = pinned_free_.find(cls);
    if (it != pinned_free_.end()) {
      void *p = it->second;
      pinned_free_.erase(it);
      return p;
    }
  }
  void *p = nullptr;
  cuda_check(cudaHostAlloc(&p, cls, cudaHostAllocPortable), "cudaHostAlloc");
  return p;
}
void Server::unpin(void *p, size_t bytes) {
  pinned_free_.emplace(pinned_class(bytes), p);  // caller holds mu_
}

int64_t Server::submit(const Request &rq) {
  if (rq.kind < kReqForward || rq.kind > kReqNorm) throw Error(kInvalidArgument, "unknown request kind");
  const int64_t need = request_bytes(rq);
  const Coverage &c = coverage(rq.coverage);
  const bool fwd = rq.kind == kReqForward || rq.kind == kReqForwardAdjoint;
  const bool adj = rq.kind == kReqAdjoint || rq.kind == kReqForwardAdjoint;
  if (fwd && (!rq.x_in || (c.M > 0 && !rq.vis_out)))
    throw Error(kInvalidArgument, "a forward request needs x_in and vis_out");
  if (rq.kind == kReqAdjoint && c.M > 0 && !rq.vis_in)
    throw Error(kInvalidArgument, "an adjoint request needs vis_in");
  if (adj && !rq.x_out) throw Error(kInvalidArgument, "an adjoint request needs x_out");
  if (rq.kind == kReqNorm && rq.iters < 1) throw Error(kInvalidArgument, "iters must be >= 1");
  std::shared_ptr<Job> j(new Job);
  j->server = this;
  j->rq = rq;
  j->bytes = need;
  j->t_submit = Clock::now();
  switch (rq.kind) {
    case kReqForward: j->in_bytes = 16 * size_t(c.N); j->out_bytes = 16 * size_t(c.M); break;
    case kReqAdjoint: j->in_bytes = 16 * size_t(c.M); j->out_bytes = 16 * size_t(c.N); break;
    case kReqForwardAdjoint:
      j->in_bytes = 16 * size_t(c.N);
      j->out_bytes = 16 * size_t(c.M + c.N);
      break;
    default: j->in_bytes = 0; j->out_bytes = sizeof(double) * size_t(rq.iters); break;
  }
  if (j->in_bytes) {
    j->host_in = pinned(j->in_bytes);
    copy_bytes(j->host_in, fwd ? rq.x_in : rq.vis_in, j->in_bytes);
  }
  if (j->out_bytes) j->host_out = pinned(j->out_bytes);
  int64_t ticket;
  {
    std::lock_guard<std::mutex> lk(mu_);
    ticket = next_ticket_++;
    j->ticket = ticket;
    jobs_[ticket] = j;
    ++stats_.submitted;
    if (need > cfg_.hbm_budget) {
      j->status = kRejected;
      j->done = true;
      j->t_admit = j->t_done = j->t_submit;
      ++stats_.rejected;
    } else {
      pending_.push_back(j);
      dirty_ = true;
    }
  }
  cv_.notify_one();
  done_cv_.notify_all();
  return ticket;
}

void CUDART_CB Server::on_done(void *p) {
  Job *j = static_cast<Job *>(p);
  Server *s = j->server;
  {
    std::lock_guard<std::mutex> lk(s->mu_);
    j->t_done = Clock::now();
    s->completed_.push_back(j);
    s->dirty_ = true;
  }
  s->cv_.notify_one();
}

void Server::loop() {
  cudaSetDevice(cfg_.device);
  std::unique_lock<std::mutex> lk(mu_);
  for (;;) {
    cv_.wait(lk, [&] { return dirty_; });
    dirty_ = false;
    while (!completed_.empty()) {
      Job *j = completed_.front();
      completed_.pop_front();
      finish(*j);
    }
    // Admission: first come first served, but a request that fits may
    // overtake a head that does not (a bounded number of times).  Slots and
    // bytes are reserved under the lock; the launches are enqueued without
    // it, so submit() and completions are not held up by a long request.
    std::vector<Job *> admitted;
    auto it = pending_.begin();
    // the head waits for a slot of its class (not for the budget): other
    // requests passing it then do not count as overtakes
    bool head_class_blocked = false;
    while (it != pending_.end()) {
      Job &j = **it;
      // norm requests: a free long slot only; others: a free short slot,
      // else a free long slot
      const bool long_job = j.rq.kind == kReqNorm;
      Slot *free = nullptr;
      for (int pass = 0; pass < 2 && !free; ++pass)
        for (auto &s : slots_)
          if (!s->busy && s->long_slot == (long_job || pass == 1)) {
            free = s.get();
            break;
          }
      if (!free) {
        bool any = false;
        for (auto &s : slots_) any |= !s->busy;
        if (!any) break;
        // only slots of the other class are free: look further down the queue
        if (it == pending_.begin()) head_class_blocked = true;
        if (!head_class_blocked && pending_.front()->overtaken >= kMaxOvertakes) break;
        ++it;
        continue;
      }
      if (bytes_in_use_ + j.bytes <= cfg_.hbm_budget) {
        if (it != pending_.begin() && !head_class_blocked) ++pending_.front()->overtaken;
        reserve(j, *free);
        admitted.push_back(&j);
        it = pending_.erase(it);
        continue;
      }
      if (pending_.front()->overtaken >= kMaxOvertakes) break;
      ++it;
    }
    for (Job *j : admitted) {
      j->slot->job = j;
      j->slot->cv.notify_one();
    }
    if (stop_ && pending_.empty() && inflight_ == 0) break;
  }
}

// A slot's enqueue thread.  The cuFFT handles are looked up under the lock
// (add_coverage inserts into the same maps); the launches are enqueued
// without it.  Requests of one coverage still enqueue one at a time (the
// operator serialises its workspace switch), those of different coverages
// in parallel.
void Server::work(Slot &slot) {
  cudaSetDevice(cfg_.device);
  std::unique_lock<std::mutex> lk(mu_);
  for (;;) {
    slot.cv.wait(lk, [&] { return slot.job != nullptr || workers_stop_; });
    if (!slot.job) break;
    Job *j = slot.job;
    slot.job = nullptr;
    cufftHandle fft = 0, cols = 0;
    try {
      const Coverage &c = coverage(j->rq.coverage);
      const int64_t key = plan_key(c.fp64, int(c.info.ftsizeu), int(c.info.ftsizev));
      fft = slot.plans.at(key);
      const auto cp = slot.col_plans.find(key);
      cols = cp == slot.col_plans.end() ? 0 : cp->second;
    } catch (...) {
      j->status = kInternal;
      j->t_done = Clock::now();
      finish(*j);
      dirty_ = true;
      cv_.notify_one();
      continue;
    }
    lk.unlock();
    const bool ok = enqueue(*j, fft, cols);
    lk.lock();
    if (!ok) {
      // nothing will call back: retire the job here and wake the scheduler
      finish(*j);
      dirty_ = true;
      cv_.notify_one();
    }
  }
}

void Server::reserve(Job &j, Slot &slot) {
  j.slot = &slot;
  j.t_admit = Clock::now();
  slot.busy = true;
  bytes_in_use_ += j.bytes;
  ++inflight_;
  stats_.bytes_peak = std::max(stats_.bytes_peak, bytes_in_use_);
  stats_.inflight_peak = std::max(stats_.inflight_peak, inflight_);
}

// Enqueues the request's copies and kernels on its slot's stream (called
// without the server lock).  Returns false if enqueueing failed; the caller
// then retires the job.
bool Server::enqueue(Job &j, cufftHandle fft, cufftHandle fft_cols) {
  const Coverage &c = coverage(j.rq.coverage);
  Slot &slot = *j.slot;
  cudaStream_t s = slot.stream;
  try {
    cuda_check(cudaMallocFromPoolAsync(&j.dev, size_t(j.bytes), pool_, s), "request memory");
    char *p = static_cast<char *>(j.dev);
    auto take = [&](size_t b) {
      char *q = p;
      p += up256(b);
      return static_cast<void *>(q);
    };
    Workspace ws;
    ws.pad = take(size_t(c.ws.pad));
    ws.work = take(size_t(c.ws.work));
    ws.tilebuf = take(size_t(c.ws.tilebuf));
    ws.slots = take(size_t(c.ws.slots));
    ws.fft = fft;
    ws.fft_cols = fft_cols;
    ws.stream = s;
    // the padded grid must be zero outside the image region
    cuda_check(cudaMemsetAsync(ws.pad, 0, size_t(c.ws.pad), s), "cudaMemsetAsync");
    const size_t cs = c.fp64 ? 16 : 8;
    if (j.rq.kind == kReqNorm) {
      void *x = take(cs * size_t(c.N));
      double *sq = static_cast<double *>(take(sizeof(double) * j.rq.iters));
      double *partial = static_cast<double *>(take(sizeof(double) * kNormBlocks));
      // The rounds go in kNormChunk at a time, at most two pieces in
      // flight: before enqueueing a piece this thread waits for the one two
      // pieces back.  A whole request at once (about 11 launches a round)
      // could fill the device's launch queue, and then every other
      // request's launches wait behind it; it would also hold the
      // coverage's lock for the whole enqueue.
      for (int i0 = 0, k = 0; i0 < j.rq.iters; i0 += kNormChunk, ++k) {
        if (k >= 2) cuda_check(cudaEventSynchronize(slot.chunk_ev[k & 1]), "cudaEventSynchronize");
        c.op->power_ws(x, i0, std::min(kNormChunk, j.rq.iters - i0), sq, partial, ws);
        cuda_check(cudaEventRecord(slot.chunk_ev[k & 1], s), "cudaEventRecord");
      }
      cuda_check(cudaMemcpyAsync(j.host_out, sq, sizeof(double) * j.rq.iters,
                                 cudaMemcpyDeviceToHost, s),
                 "D2H");
    } else {
      void *x128 = take(16 * size_t(c.N));
      void *y128 = take(16 * size_t(std::max<int64_t>(c.M, 1)));
      void *xc = x128, *yc = y128;
      if (!c.fp64) {
        xc = take(8 * size_t(c.N));
        yc = take(8 * size_t(std::max<int64_t>(c.M, 1)));
      }
      auto to_work = [&](void *src128, void *dst, int64_t n) {
        if (!c.fp64) cuda_check(launch_from_c128<float>(src128, dst, n, s), "convert");
      };
      auto to_c128 = [&](void *src, void *dst128, int64_t n) {
        if (!c.fp64) cuda_check(launch_to_c128<float>(src, dst128, n, s), "convert");
      };
      const bool fwd = j.rq.kind != kReqAdjoint;
      if (fwd) {
        cuda_check(cudaMemcpyAsync(x128, j.host_in, 16 * size_t(c.N), cudaMemcpyHostToDevice, s),
                   "H2D");
        to_work(x128, xc, c.N);
        c.op->forward_ws(xc, yc, ws);
      } else if (c.M > 0) {
        cuda_check(cudaMemcpyAsync(y128, j.host_in, 16 * size_t(c.M), cudaMemcpyHostToDevice, s),
                   "H2D");
        to_work(y128, yc, c.M);
      }
      if (j.rq.kind != kReqForward) {
        if (j.rq.kind == kReqAdjoint && c.M == 0)
          cuda_check(cudaMemsetAsync(yc, 0, cs, s), "cudaMemsetAsync");
        // x was read by the forward's first kernel, so its buffer takes the image
        c.op->adjoint_ws(yc, xc, ws);
      }
      char *out = static_cast<char *>(j.host_out);
      if (fwd && c.M > 0) {
        to_c128(yc, y128, c.M);
        cuda_check(cudaMemcpyAsync(out, y128, 16 * size_t(c.M), cudaMemcpyDeviceToHost, s), "D2H");
        out += 16 * size_t(c.M);
      }
      if (j.rq.kind != kReqForward) {
        to_c128(xc, x128, c.N);
        cuda_check(cudaMemcpyAsync(out, x128, 16 * size_t(c.N), cudaMemcpyDeviceToHost, s), "D2H");
      }
    }
    cuda_check(cudaLaunchHostFunc(s, &Server::on_done, &j), "cudaLaunchHostFunc");
    return true;
  } catch (const Error &e) {
    // Nothing will call back: the caller retires the job.  Work already
    // enqueued finishes before the stream-ordered free.
    j.status = int(e.status);
  } catch (const std::bad_alloc &) {
    j.status = kOutOfMemory;
  } catch (...) {
    j.status = kInternal;
  }
  j.t_done = Clock::now();
  return false;
}

void Server::finish(Job &j) {
  Slot &slot = *j.slot;
  if (j.dev) cudaFreeAsync(j.dev, slot.stream);
  j.dev = nullptr;
  slot.busy = false;
  bytes_in_use_ -= j.bytes;
  --inflight_;
  const Coverage &c = coverage(j.rq.coverage);
  if (j.status == kOk && j.rq.kind == kReqNorm) {
    // the single-operator stopping rule on the recorded estimates
    const double *sq = static_cast<const double *>(j.host_out);
    double old_value = 0;
    for (int i = 0; i < j.rq.iters; ++i) {
      const double value = std::sqrt(sq[i]);
      j.iterations = i + 1;
      if (!(value > 0)) {
        j.status = kNormNotPositive;
        break;
      }
      if (j.rq.tol * j.rq.tol > std::abs(old_value - value) / old_value) {
        old_value = value;
        break;
      }
      old_value = value;
    }
    j.norm = std::sqrt(old_value);
  }
  if (j.status == kOk) {
    ++stats_.completed;
    const double passes = j.rq.kind == kReqNorm ? 2.0 * j.rq.iters
                          : j.rq.kind == kReqForwardAdjoint ? 2.0 : 1.0;
    stats_.visibility_passes += passes * double(c.M);
    latencies_.push_back(ms_between(j.t_submit, j.t_done));
  } else {
    ++stats_.failed;
  }
  j.done = true;
  done_cv_.notify_all();
}

bool Server::wait(int64_t ticket, double timeout_s, RequestResult *out) {
  std::shared_ptr<Job> j;
  {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = jobs_.find(ticket);
    if (it == jobs_.end()) throw Error(kInvalidArgument, "unknown ticket");
    j = it->second;
    auto ready = [&] { return j->done; };
    if (timeout_s < 0)
      done_cv_.wait(lk, ready);
    else if (!done_cv_.wait_for(lk, std::chrono::duration<double>(timeout_s), ready))
      return false;
    jobs_.erase(ticket);
  }
  const Coverage &c = coverage(j->rq.coverage);
  if (j->status == kOk && j->rq.kind != kReqNorm) {
    const char *src = static_cast<const char *>(j->host_out);
    if (j->rq.kind != kReqAdjoint && c.M > 0) {
      copy_bytes(j->rq.vis_out, src, 16 * size_t(c.M));
      src += 16 * size_t(c.M);
    }
    if (j->rq.kind != kReqForward) copy_bytes(j->rq.x_out, src, 16 * size_t(c.N));
  }
  if (out) {
    out->status = j->status;
    out->norm = j->norm;
    out->iterations = j->iterations;
    out->queue_ms = ms_between(j->t_submit, j->t_admit);
    out->run_ms = ms_between(j->t_admit, j->t_done);
    out->latency_ms = ms_between(j->t_submit, j->t_done);
    out->device_bytes = j->bytes;
  }
  std::lock_guard<std::mutex> lk(mu_);
  if (j->host_in) unpin(j->host_in, j->in_bytes);
  if (j->host_out) unpin(j->host_out, j->out_bytes);
  j->host_in = j->host_out = nullptr;
  return true;
}

ServerStats Server::stats() const {
  std::lock_guard<std::mutex> lk(mu_);
  ServerStats s = stats_;
  if (!latencies_.empty()) {
    std::vector<double> v = latencies_;
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) {
      // nearest-rank percentile
      const size_t k = size_t(std::ceil(q * double(v.size())));
      return v[std::min(v.size() - 1, k == 0 ? 0 : k - 1)];
    };
    s.latency_p50_ms = pct(0.50);
    s.latency_p99_ms = pct(0.99);
    double sum = 0;
    for (double x : v) sum += x;
    s.latency_mean_ms = sum / double(v.size());
  }
  return s;
}

}  // namespace pg
