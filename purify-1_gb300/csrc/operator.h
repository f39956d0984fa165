// Host side of the GB300 measurement operator: device state of one coverage,
// cuFFT plan, and the apply / power-method drivers.
#pragma once
#include <cuda_runtime_api.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>

#include "pg_types.h"

namespace pg {

class Error : public std::runtime_error {
 public:
  Error(Status s, const std::string &msg) : std::runtime_error(msg), status(s) {}
  Status status;
};

// Throws pg::Error on a CUDA failure, naming the call.
void cuda_check(cudaError_t e, const char *what);

struct OperatorConfig {
  const double *u = nullptr, *v = nullptr, *w = nullptr;
  const double *weights = nullptr;  // interleaved complex, or null
  int64_t M = 0;
  int imsizey = 0, imsizex = 0;
  double oversample_ratio = 2.0;
  int power_iters = 100;
  double power_tol = 1e-4;
  int kernel = kKB;
  int Ju = 4, Jv = 4;
  bool w_term = false;
  int Jw = 6;
  const int32_t *jw_rows = nullptr;  // per-row w-support, or null for Jw
  double cellx = 1.0, celly = 1.0;
  bool fp64 = false;
  int device = 0;
  // tuning (defaults chosen by the autotuner's table when left at 0)
  int threads = 0;
  int max_per_item = 0;
  int tile = 0;
  // 1: degrid/grid read and write caller-ordered visibilities directly;
  // 0: through a slot-ordered buffer and separate gather kernels;
  // -1: default (direct for the forward, gather for the adjoint).
  int fused_permute = -1;
  // cells per work item along each axis: 0 picks 2 for complex<float> with
  // J <= kMaxGroupJ (2 x 2 groups of base cells, a (J + 1)^2 block), else 1
  int cell_group = 0;
  // most items of one bank class per batch (0: the planner's default)
  int class_cap = 0;
  // 1: the forward's caller-ordered output is stored at L2 evict-last priority
  int keep_store = 0;
  // column transform of the fused FFT path (FP32, power-of-two grid):
  // 0: the library's column pass where it applies (grid height <= 2048),
  // 1: cuFFT's strided column plan
  int fft_columns = 0;
  // G^H of Phi^H: 1 = the column walk (plan.h WalkPlan) where it applies,
  // 0 = the work-item kernel.  The walk flushes a third of the shared-memory
  // traffic but runs 2.2x the visibility steps on the 10^7 workload (a
  // column lasts as long as its fullest row), and measured slower there.
  int grid_walk = 0;
  // G^H G of the normal operator: 1 = normal_kernel's one pass where it
  // applies, 2 = degrid then grid through the slot buffer, 0 = the default
  // (one pass for J < 6).  The one pass evaluates the taps once and keeps
  // no slot vector, but holds two J x J register blocks (194 registers at
  // J = 6, where it measured slower).
  int normal_pass = 0;
};

// A plan fraction t + d (see PlanRequest::group) in precision `real`, kept
// below d + 1 after rounding.
template <typename real>
real fraction_in_cell(double x);

// S(j, i) = 1 / (ftv(y0 + j + 0.5) ftu(x0 + i + 0.5)) for the kernel, as
// row-major imsizey x imsizex reals.
void correction_factors(int kernel, int Ju, int Jv, int imsizey, int imsizex, double os,
                        double *S);

struct OperatorInfo {
  int64_t M = 0;
  int imsizey = 0, imsizex = 0, ftsizev = 0, ftsizeu = 0, Ju = 0, Jv = 0;
  bool fp64 = false;
  int kernel = 0;
  bool w_term = false;
  int64_t nnz = 0, occupied_cells = 0, work_items = 0, tasks = 0, device_bytes = 0;
  double kernel_fit_error = 0, norm = 1;
  int device = 0;
  int64_t slots = 0, window_cells = 0, factor_values = 0, cell_group = 1;
  int64_t walk_tasks = 0, walk_steps = 0;
};

// Scratch of one apply held outside the operator, so that several applies of
// one coverage can be in flight at once on different streams.
struct Workspace {
  void *pad = nullptr;      // Nv x Nu complex, zero outside the image region
  void *work = nullptr;     // Nv x Nu complex
  void *tilebuf = nullptr;  // accumulation windows of the tasks
  void *slots = nullptr;    // slot-ordered visibilities
  int fft = 0;              // cuFFT plan (cufftHandle) of Nv x Nu, bound to `stream`
  // FP32 grids with power-of-two widths: a cuFFT plan of the Nu columns
  // (length Nv, stride Nu), bound to `stream`; with it the operator runs the
  // fused row passes (fft_kernels.h) instead of pad + 2-D FFT + crop.
  int fft_cols = 0;
  cudaStream_t stream = nullptr;
  bool unit_norm = false;   // apply Phi' (norm 1) instead of Phi
};
struct WorkspaceSizes {
  int64_t pad = 0, work = 0, tilebuf = 0, slots = 0;  // bytes
};

class Operator {
 public:
  static std::unique_ptr<Operator> create(const OperatorConfig &cfg);
  virtual ~Operator() = default;

  // Device buffers of the operator's precision; ordered after `stream`.
  virtual void forward(const void *x, void *y, cudaStream_t stream) = 0;
  virtual void adjoint(const void *y, void *x, cudaStream_t stream) = 0;
  // Phi^H Phi x with the visibilities kept in slot order between the two
  // halves (no caller-order permutation): the combined degrid/grid operator.
  virtual void normal(const void *x, void *out, cudaStream_t stream) = 0;
  // G and G^H alone (no correction, padding or FFT).
  virtual void degrid(const void *grid, void *vis, cudaStream_t stream) = 0;
  virtual void grid(const void *vis, void *grid, cudaStream_t stream) = 0;
  // G^H with its scratch in the library's fixed device array (no allocation).
  virtual void grid_no_alloc(const void *vis, void *grid, cudaStream_t stream) = 0;
  virtual int64_t no_alloc_bytes() const = 0;
  // Host complex<double> buffers; synchronous.
  virtual void forward_host(const double *x, double *y) = 0;
  virtual void adjoint_host(const double *y, double *x) = 0;
  // Sets the norm to ||Phi'|| from the power method and returns it.
  virtual double power_method(int iters, double tol) = 0;
  virtual void set_norm(double norm) = 0;
  virtual double norm() const = 0;
  virtual OperatorInfo info() const = 0;
  // Stage timing (see purify_gb300_stage_timing).
  static constexpr int kStages = 9;
  virtual void set_stage_timing(bool on) = 0;
  virtual void stage_times(double *total_ms, int64_t *launches) = 0;
  // Applies on a caller's workspace: enqueued on ws.stream only (no wait on
  // the operator's own stream), coverage state read-only.
  virtual WorkspaceSizes workspace_sizes() const = 0;
  virtual void forward_ws(const void *x, void *y, const Workspace &ws) = 0;
  virtual void adjoint_ws(const void *y, void *x, const Workspace &ws) = 0;
  // Power-method rounds first ... first+count-1 of Phi'^H Phi' on x (N
  // complex scratch), the normalisation on the device; round 0 starts from
  // the normalised all-ones image.  sq[i] (device) receives ||x||^2 of round
  // i, partial is kNormBlocks doubles.  Rounds may be enqueued in pieces.
  virtual void power_ws(void *x, int first, int count, double *sq, double *partial,
                        const Workspace &ws) = 0;
  // True when the applies need Workspace::fft_cols (a cuFFT column plan).
  virtual bool needs_column_plan() const = 0;
};

}  // namespace pg
