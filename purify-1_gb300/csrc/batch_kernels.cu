// Grouped (multi-channel) launches: one grid over the tasks or pixels of
// several operators.  The degrid / grid kernels read each task's operator
// arguments from a device table indexed by Task::channel; the element-wise
// kernels take one CTA row (blockIdx.y) per channel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "device_kernels.h"
#include "gridding_device.cuh"

namespace pg {
namespace {
using namespace dev;

// The element-wise grouped kernels run over a block map: block b works on
// channel map[b].x, its block map[b].y, so no block is idle whatever the
// spread of channel sizes.
template <typename real>
__global__ void fold_group_kernel(const FoldArgs *__restrict__ folds, const int2 *__restrict__ map) {
  const int2 m = map[blockIdx.x];
  fold_tile<real>(folds[m.x], m.y);
}

template <typename real>
__global__ void pad_group_kernel(const ChannelIO<real> *__restrict__ chans,
                                 const int2 *__restrict__ map) {
  const int2 m = map[blockIdx.x];
  const ChannelIO<real> &c = chans[m.x];
  const int64_t idx = int64_t(m.y) * blockDim.x + threadIdx.x;
  if (idx >= int64_t(c.Nx) * c.Ny) return;
  const int j = int(idx / c.Nx), i = int(idx - int64_t(j) * c.Nx);
  const real s = c.su[i] * c.sv[j];
  const cplx<real> v = static_cast<const cplx<real> *>(c.x_in)[idx];
  static_cast<cplx<real> *>(c.pad)[int64_t(c.y0 + j) * (c.ld ? c.ld : c.Nu) + c.x0 + i] =
      cplx<real>{s * v.x, s * v.y};
}
template <typename real>
__global__ void crop_group_kernel(const ChannelIO<real> *__restrict__ chans,
                                  const int2 *__restrict__ map) {
  const int2 m = map[blockIdx.x];
  const ChannelIO<real> &c = chans[m.x];
  const int64_t idx = int64_t(m.y) * blockDim.x + threadIdx.x;
  if (idx >= int64_t(c.Nx) * c.Ny) return;
  const int j = int(idx / c.Nx), i = int(idx - int64_t(j) * c.Nx);
  const real s = c.su[i] * c.sv[j];
  const cplx<real> v =
      static_cast<const cplx<real> *>(c.work)[int64_t(c.y0 + j) * (c.ld ? c.ld : c.Nu) + c.x0 + i];
  static_cast<cplx<real> *>(c.x_out)[idx] = cplx<real>{s * v.x, s * v.y};
}
// slots[s] = in[slot_user[s]] (0 for null slots): a block covers 4 * 256
// consecutive slots, four gathers in flight per thread.
template <typename real>
__global__ void expand_group_kernel(const ChannelIO<real> *__restrict__ chans,
                                    const int2 *__restrict__ map) {
  const int2 mm = map[blockIdx.x];
  const ChannelIO<real> &c = chans[mm.x];
  const cplx<real> *in = static_cast<const cplx<real> *>(c.vis_in);
  cplx<real> *slots = static_cast<cplx<real> *>(c.slots);
  const int64_t s0 = int64_t(mm.y) * kGroupSlots + threadIdx.x;
  int32_t m[4];
  cplx<real> v[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) m[r] = s0 + r * 256 < c.S ? __ldcs(c.slot_user + s0 + r * 256) : -1;
#pragma unroll
  for (int r = 0; r < 4; ++r) v[r] = m[r] >= 0 ? in[m[r]] : cplx<real>{0, 0};
  if (c.w_slot) {
    // conj(w) v: G^H holds the conjugated entries of G
    const cplx<real> *w = static_cast<const cplx<real> *>(c.w_slot);
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (s0 + r * 256 < c.S) {
        const cplx<real> a = __ldcs(w + s0 + r * 256);
        v[r] = cplx<real>{a.x * v[r].x + a.y * v[r].y, a.x * v[r].y - a.y * v[r].x};
      }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
    if (s0 + r * 256 < c.S) slots[s0 + r * 256] = v[r];
}
// vis_out[m] <- vis_out[m] w_vis[m]: a block covers 4 * 256 consecutive
// caller-ordered visibilities of a channel with weights.
template <typename real>
__global__ void weigh_vis_group_kernel(const ChannelIO<real> *__restrict__ chans,
                                       const int2 *__restrict__ map) {
  const int2 mm = map[blockIdx.x];
  const ChannelIO<real> &c = chans[mm.x];
  cplx<real> *vis = static_cast<cplx<real> *>(c.vis_out);
  const cplx<real> *w = static_cast<const cplx<real> *>(c.w_vis);
  const int64_t m0 = int64_t(mm.y) * kGroupSlots + threadIdx.x;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int64_t m = m0 + r * 256;
    if (m < c.M) {
      const cplx<real> a = vis[m], b = __ldcs(w + m);
      vis[m] = cplx<real>{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
    }
  }
}

// Per-channel FP64 |x|^2 of the adjoint output, with the same fixed
// reduction shape as the single-operator norm (kNormBlocks blocks of 256
// threads, then one block over the partials), so each channel's sum does not
// depend on the batch.
template <typename real>
__global__ void sq_norm_group_partial(const ChannelIO<real> *__restrict__ chans,
                                      double *__restrict__ partial) {
  const ChannelIO<real> &c = chans[blockIdx.y];
  const cplx<real> *x = static_cast<const cplx<real> *>(c.x_out);
  const int64_t n = int64_t(c.Nx) * c.Ny;
  __shared__ double red[256];
  double s = 0;
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x) {
    const cplx<real> v = x[k];
    s += double(v.x) * double(v.x) + double(v.y) * double(v.y);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[size_t(blockIdx.y) * gridDim.x + blockIdx.x] = red[0];
}
__global__ void sq_norm_group_final(const double *__restrict__ partial, int n,
                                    double *__restrict__ out) {
  __shared__ double red[kNormBlocks];
  red[threadIdx.x] = threadIdx.x < n ? partial[size_t(blockIdx.x) * n + threadIdx.x] : 0.0;
  __syncthreads();
  for (int w = kNormBlocks / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}
// x_out of channel c <- x_out * inv[c].
template <typename real>
__global__ void scale_group_kernel(const ChannelIO<real> *__restrict__ chans,
                                   const int2 *__restrict__ map, const double *__restrict__ inv) {
  const int2 m = map[blockIdx.x];
  const ChannelIO<real> &c = chans[m.x];
  const int64_t k = int64_t(m.y) * blockDim.x + threadIdx.x;
  if (k >= int64_t(c.Nx) * c.Ny) return;
  cplx<real> *x = static_cast<cplx<real> *>(c.x_out);
  const real s = real(inv[m.x]);
  cplx<real> w = x[k];
  w.x *= s;
  w.y *= s;
  x[k] = w;
}

}  // namespace

template <typename real>
cudaError_t launch_degrid_group(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                                int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                                bool user, cudaStream_t s) {
  const size_t smem =
      degrid_smem_bytes(sizeof(real), J, win_rows, win_cols, shape, user, a.group_cells,
                        poly_nsub(poly));
  ApplyArgs<real> b = a;
  b.win_bytes = int(window_bytes(sizeof(real), win_rows, win_cols, shape, false, a.group_cells));
  b.stage_bytes = int(stage_bytes(sizeof(real), J, user));
  return launch_apply<real, true>(true, b, poly, J, ntasks, smem, shape.threads, s);
}
template <typename real>
cudaError_t launch_grid_group(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                              int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                              bool user, cudaStream_t s) {
  const size_t smem = grid_smem_bytes(sizeof(real), J, win_rows, win_cols, shape, user,
                                      a.group_cells, poly_nsub(poly));
  ApplyArgs<real> b = a;
  b.win_bytes = int(window_bytes(sizeof(real), win_rows, win_cols, shape, true, a.group_cells));
  return launch_apply<real, true>(false, b, poly, J, ntasks, smem, shape.threads, s);
}

template <typename real>
cudaError_t launch_fold_group(const FoldArgs *folds, const int2 *map, int nblocks, cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  fold_group_kernel<real><<<nblocks, dim3(32, 8), 0, s>>>(folds, map);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_pad_group(const ChannelIO<real> *chans, const int2 *map, int nblocks,
                             cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  pad_group_kernel<real><<<nblocks, kGroupPixels, 0, s>>>(chans, map);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_crop_group(const ChannelIO<real> *chans, const int2 *map, int nblocks,
                              cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  crop_group_kernel<real><<<nblocks, kGroupPixels, 0, s>>>(chans, map);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_expand_group(const ChannelIO<real> *chans, const int2 *map, int nblocks,
                                cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  expand_group_kernel<real><<<nblocks, 256, 0, s>>>(chans, map);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_weigh_vis_group(const ChannelIO<real> *chans, const int2 *map, int nblocks,
                                   cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  weigh_vis_group_kernel<real><<<nblocks, 256, 0, s>>>(chans, map);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_sq_norm_group(const ChannelIO<real> *chans, int nch, double *partial,
                                 double *out, cudaStream_t s) {
  if (nch == 0) return cudaSuccess;
  sq_norm_group_partial<real><<<dim3(kNormBlocks, nch), 256, 0, s>>>(chans, partial);
  sq_norm_group_final<<<nch, kNormBlocks, 0, s>>>(partial, kNormBlocks, out);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_scale_group(const ChannelIO<real> *chans, const int2 *map, int nblocks,
                               const double *inv, cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  scale_group_kernel<real><<<nblocks, kGroupPixels, 0, s>>>(chans, map, inv);
  return cudaGetLastError();
}

#define PG_INSTANTIATE_GROUP(real)                                                               \
  template cudaError_t launch_degrid_group<real>(const ApplyArgs<real> &, const PolyTable<real> &,  \
                                                 int, int, int, int, const LaunchShape &, bool,    \
                                                 cudaStream_t);                                    \
  template cudaError_t launch_grid_group<real>(const ApplyArgs<real> &, const PolyTable<real> &,    \
                                               int, int, int, int, const LaunchShape &, bool,      \
                                               cudaStream_t);                                      \
  template cudaError_t launch_fold_group<real>(const FoldArgs *, const int2 *, int, cudaStream_t);  \
  template cudaError_t launch_pad_group<real>(const ChannelIO<real> *, const int2 *, int,          \
                                              cudaStream_t);                                       \
  template cudaError_t launch_crop_group<real>(const ChannelIO<real> *, const int2 *, int,         \
                                               cudaStream_t);                                      \
  template cudaError_t launch_expand_group<real>(const ChannelIO<real> *, const int2 *, int,       \
                                                 cudaStream_t);                                    \
  template cudaError_t launch_weigh_vis_group<real>(const ChannelIO<real> *, const int2 *, int,    \
                                                    cudaStream_t);                                 \
  template cudaError_t launch_sq_norm_group<real>(const ChannelIO<real> *, int, double *, double *, \
                                                  cudaStream_t);                                   \
  template cudaError_t launch_scale_group<real>(const ChannelIO<real> *, const int2 *, int,        \
                                                const double *, cudaStream_t);

PG_INSTANTIATE_GROUP(float)
PG_INSTANTIATE_GROUP(double)

}  // namespace pg
