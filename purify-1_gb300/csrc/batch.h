// Multi-channel batch: many measurement operators (channels or snapshots with
// their own coverage and image size, one kernel and support) applied
// together.  Each Phi / Phi^H step is a handful of grouped launches -- one
// degrid and one grid launch over the tasks of every channel, element-wise
// kernels with one CTA row per channel, cuFFT batched per image size --
// captured once into a CUDA graph and replayed.
#pragma once
#include <cuda_runtime_api.h>

#include <complex>
#include <cstdint>
#include <memory>
#include <vector>

#include "operator.h"

namespace pg {

struct ChannelSpec {
  const double *u = nullptr, *v = nullptr;
  const std::complex<double> *weights = nullptr;  // or null for ones
  int64_t M = 0;
  int imsizey = 0, imsizex = 0;
};

struct BatchConfig {
  std::vector<ChannelSpec> channels;
  double oversample_ratio = 2.0;
  int kernel = kKB;
  int J = 4;
  bool fp64 = false;
  int device = 0;
  int threads = 128;        // CTA size of both gridding kernels, unless set below
  int degrid_threads = 0;   // 0: threads
  int grid_threads = 0;     // 0: threads
  int max_per_item = 16;
  int tile = kTile;
  int cell_group = 1;       // cells per work item along each axis (1, or 2 for FP32, J <= 6)
  // column transforms of the fused size groups: 0 = launch_fft_cols where it
  // applies, 1 = a strided cuFFT plan
  int fft_columns = 0;
};

struct BatchInfo {
  int channels = 0;
  int64_t visibilities = 0, pixels = 0, tasks = 0, device_bytes = 0;
  int size_groups = 0;
  int win_rows = 0, win_cols = 0;  // largest task window over the channels
};

class Batch {
 public:
  static std::unique_ptr<Batch> create(const BatchConfig &cfg);
  virtual ~Batch() = default;
  // Device pointers (one per channel) of the forward input images, the
  // visibilities (forward output, adjoint input) and the adjoint output
  // images; complex of the batch's precision.  Stream-ordered on `stream`.
  virtual void bind(const void *const *x_in, void *const *vis, void *const *x_out,
                    cudaStream_t stream) = 0;
  // directions: 1 forward, 2 adjoint, 3 both (forward first).
  virtual void apply(int directions, cudaStream_t stream) = 0;
  // Per-channel operator norms: Phi_c = G F Z S / norm_c.
  virtual void set_norms(const double *norms) = 0;
  virtual void get_norms(double *norms) const = 0;
  // Power method of every channel at once (the single-operator rule per
  // channel); sets the norms and writes them to `norms` if not null.  The
  // bound buffers are kept; the batch's own stream is synchronised.
  virtual void power_method(int iters, double tol, double *norms) = 0;
  virtual BatchInfo info() const = 0;
  // CTA sizes of the grouped degrid / grid launches; drops recorded graphs.
  virtual void set_launch_shapes(int degrid_threads, int grid_threads) = 0;
  // Average device milliseconds of one replay of `directions` over `reps`
  // replays (after two untimed ones), on the batch's own buffers; the bound
  // buffers are kept.  directions 8 / 16 time the grouped degrid / grid
  // launch alone.
  virtual double time_apply(int directions, int reps) = 0;
};

// Launch and layout parameters of a batch.
struct BatchTuning {
  int tile = kTile, max_per_item = 16, degrid_threads = 128, grid_threads = 128;
  int cell_group = 1;
  int fft_columns = 0;
};

// Picks the uv tile edge, the work-item shape (single cells or 2 x 2 groups)
// and the CTA sizes of the two gridding kernels for this batch by timing
// candidates on the GPU: a sample of up to eight channels (evenly spaced in
// visibility count) is planned for each tile edge and item shape, and each
// plan is timed with each CTA size, forward and adjoint apart.
// Results are cached per process, keyed by precision, kernel, support,
// oversampling and the sample's sizes.
BatchTuning autotune_batch(const BatchConfig &cfg);

}  // namespace pg
