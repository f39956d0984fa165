// Host-callable launchers of the sm_103a kernels.  Plain C++ declarations so
// that host translation units compiled by g++ can call them.
#pragma once
#include <cuda_runtime_api.h>

#include <cstddef>
#include <cstdint>

#include "pg_types.h"

namespace pg {

// Pointers and sizes of one coverage plus the I/O buffers of one apply.
// Complex arrays hold interleaved (re, im) pairs of `real`.  Visibility
// vectors here are in slot order (see plan.h).
template <typename real>
struct ApplyArgs {
  const void *grid = nullptr;       // degrid input: Nv x Nu complex
  void *tilebuf = nullptr;          // grid output: one window per task
  const Task *tasks = nullptr;
  const int2 *batches = nullptr;    // {first slot, kmax}
  const int32_t *lane_code = nullptr;  // item_pack per batch lane
  const void *frac = nullptr;       // S x (t_u, t_v); sign of t_u = phase flip if unit weights
  const void *weight = nullptr;     // S complex weights with the flip folded in, or null
  void *slot_out = nullptr;         // degrid output, S complex
  const void *slot_in = nullptr;    // grid input, S complex
  // When set, visibilities are read / written in caller order directly:
  // slot s holds visibility slot_user[s] (-1 = null slot), slot_out and
  // slot_in then point at caller-ordered M-vectors.
  const int32_t *slot_user = nullptr;
  int Nu = 0, Nv = 0;
  int64_t slot_stride = 0;          // complex elements per tilebuf slot
  int win_bytes = 0;  // set by the launchers: shared bytes before the batch headers
};

struct LaunchShape {
  int threads = 128;  // 32 x warps per CTA
};

// Largest dynamic shared memory a launch of the given shape needs, in bytes.
size_t degrid_smem_bytes(int precision_bytes, int J, int win_rows, int win_cols,
                         const LaunchShape &shape);
size_t grid_smem_bytes(int precision_bytes, int J, int win_rows, int win_cols,
                       const LaunchShape &shape);

// G: tiles of the grid -> visibilities.
template <typename real>
cudaError_t launch_degrid(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                          int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                          cudaStream_t s);
// G^H, first half: visibilities -> one accumulated window per task.
template <typename real>
cudaError_t launch_grid(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                        int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                        cudaStream_t s);

// G^H, second half: sums the task windows that cover each grid cell, in a
// fixed order, into the grid.
struct FoldArgs {
  const void *tilebuf;
  int64_t slot_stride;
  const int32_t *tile_tasks;         // ntiles + 1
  const int32_t *tu_start, *tv_start;  // ntu + 1, ntv + 1
  const int32_t *tu_of, *tv_of;      // Nu, Nv
  int ntu, ntv, Ju, Jv, Nu, Nv;
  void *grid;
};
template <typename real>
cudaError_t launch_fold(const FoldArgs &f, cudaStream_t s);

// Z S: scaled gridding correction and zero padding.  su[i] sv[j] x[j Nx + i]
// lands at grid[(y0 + j) Nu + x0 + i]; other grid cells are left untouched.
template <typename real>
cudaError_t launch_pad(const void *x, const real *su, const real *sv, void *grid, int Nx, int Ny,
                       int Nu, int x0, int y0, cudaStream_t s);
// S^H Z^H: crop and scaled correction.
template <typename real>
cudaError_t launch_crop(const void *grid, const real *su, const real *sv, void *x, int Nx, int Ny,
                        int Nu, int x0, int y0, cudaStream_t s);

// Caller order <-> slot order.  compact: out[m] = slots[user_slot[m]], m < M.
// expand: slots[s] = in[slot_user[s]] (0 where slot_user[s] < 0), s < S.
template <typename real>
cudaError_t launch_compact(const void *slots, const int32_t *user_slot, void *out, int64_t M,
                           cudaStream_t s);
template <typename real>
cudaError_t launch_expand(const void *in, const int32_t *slot_user, void *slots, int64_t S,
                          cudaStream_t s);

// complex<double> <-> complex<real> conversion of n values.
template <typename real>
cudaError_t launch_from_c128(const void *src, void *dst, int64_t n, cudaStream_t s);
template <typename real>
cudaError_t launch_to_c128(const void *src, void *dst, int64_t n, cudaStream_t s);

// Deterministic FP64 sum of |x|^2 over n complex values into *out (device).
// `partial` must hold kNormBlocks doubles.
constexpr int kNormBlocks = 512;
template <typename real>
cudaError_t launch_sq_norm(const void *x, int64_t n, double *partial, double *out,
                           cudaStream_t s);
// x <- x * scale.
template <typename real>
cudaError_t launch_scale(void *x, int64_t n, double scale, cudaStream_t s);
// x <- value (complex, real part only).
template <typename real>
cudaError_t launch_fill(void *x, int64_t n, double value, cudaStream_t s);

}  // namespace pg
