// Host-callable launchers of the w-projection gridding kernels.
#pragma once
#include <cuda_runtime_api.h>

#include <cstddef>
#include <cstdint>

#include "pg_types.h"

namespace pg {

// Largest w-projection support (taps per axis) one warp handles.
constexpr int kMaxWSupport = 32;

template <typename real>
struct WArgs {
  const void *grid = nullptr;      // degrid input, Nv x Nu complex
  void *tilebuf = nullptr;         // grid output: one window per task
  const Task *tasks = nullptr;     // batch_begin / batch_end = visibility range
  const int32_t *order = nullptr;  // CTA b runs task order[b], or task b when null
  const int32_t *code = nullptr;   // per visibility: lp | lq << 8 | S << 16
  const int64_t *factor = nullptr; // per visibility: first factor (complex index)
  const void *factors = nullptr;   // complex factors A_0..A_2, B_0..B_2 per row
  const void *weight = nullptr;    // per visibility, complex, phase sign folded in
  void *slot_out = nullptr;        // degrid output in plan order
  const void *slot_in = nullptr;   // grid input in plan order
  const WChunk *chunks = nullptr;  // staging chunks (wplan.h)
  const int32_t *task_chunk = nullptr;
  int chunk_values = 0;
  int Nu = 0, Nv = 0, Smax = 0;
  int64_t slot_stride = 0;
  int win_bytes = 0;               // set by the launchers
};

// Both kernels run 256 threads per CTA with one window per CTA and the row
// data staged chunk by chunk (WArgs::chunks).
template <typename real>
size_t wdegrid_smem_bytes(int win_rows, int win_cols, int chunk_values);
template <typename real>
size_t wgrid_smem_bytes(int win_rows, int win_cols, int chunk_values);
template <typename real>
cudaError_t launch_wdegrid(const WArgs<real> &a, int ntasks, int win_rows, int win_cols,
                           cudaStream_t s);
template <typename real>
cudaError_t launch_wgrid(const WArgs<real> &a, int ntasks, int win_rows, int win_cols,
                         cudaStream_t s);

}  // namespace pg
