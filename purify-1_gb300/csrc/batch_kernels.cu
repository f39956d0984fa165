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

template <typename real>
__global__ void fold_group_kernel(const FoldArgs *__restrict__ folds) {
  const FoldArgs &f = folds[blockIdx.y];
  if (int(blockIdx.x) < f.ntu * f.ntv) fold_tile<real>(f, blockIdx.x);
}

template <typename real>
__global__ void pad_group_kernel(const ChannelIO<real> *__restrict__ chans) {
  const ChannelIO<real> &c = chans[blockIdx.y];
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= int64_t(c.Nx) * c.Ny) return;
  const int j = int(idx / c.Nx), i = int(idx - int64_t(j) * c.Nx);
  const real s = c.su[i] * c.sv[j];
  const cplx<real> v = static_cast<const cplx<real> *>(c.x_in)[idx];
  static_cast<cplx<real> *>(c.pad)[int64_t(c.y0 + j) * c.Nu + c.x0 + i] =
      cplx<real>{s * v.x, s * v.y};
}
template <typename real>
__global__ void crop_group_kernel(const ChannelIO<real> *__restrict__ chans) {
  const ChannelIO<real> &c = chans[blockIdx.y];
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= int64_t(c.Nx) * c.Ny) return;
  const int j = int(idx / c.Nx), i = int(idx - int64_t(j) * c.Nx);
  const real s = c.su[i] * c.sv[j];
  const cplx<real> v = static_cast<const cplx<real> *>(c.work)[int64_t(c.y0 + j) * c.Nu + c.x0 + i];
  static_cast<cplx<real> *>(c.x_out)[idx] = cplx<real>{s * v.x, s * v.y};
}
template <typename real>
__global__ void compact_group_kernel(const ChannelIO<real> *__restrict__ chans) {
  const ChannelIO<real> &c = chans[blockIdx.y];
  const cplx<real> *slots = static_cast<const cplx<real> *>(c.slots);
  cplx<real> *out = static_cast<cplx<real> *>(c.vis_out);
  for (int64_t m = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; m < c.M;
       m += int64_t(gridDim.x) * blockDim.x)
    __stcs(out + m, slots[__ldcs(c.user_slot + m)]);
}
template <typename real>
__global__ void expand_group_kernel(const ChannelIO<real> *__restrict__ chans) {
  const ChannelIO<real> &c = chans[blockIdx.y];
  const cplx<real> *in = static_cast<const cplx<real> *>(c.vis_in);
  cplx<real> *slots = static_cast<cplx<real> *>(c.slots);
  for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < c.S;
       s += int64_t(gridDim.x) * blockDim.x) {
    const int32_t m = __ldcs(c.slot_user + s);
    slots[s] = m >= 0 ? in[m] : cplx<real>{0, 0};
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
                                   const double *__restrict__ inv) {
  const ChannelIO<real> &c = chans[blockIdx.y];
  cplx<real> *x = static_cast<cplx<real> *>(c.x_out);
  const int64_t n = int64_t(c.Nx) * c.Ny;
  const real s = real(inv[blockIdx.y]);
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x) {
    cplx<real> v = x[k];
    v.x *= s;
    v.y *= s;
    x[k] = v;
  }
}

}  // namespace

template <typename real>
cudaError_t launch_degrid_group(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                                int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                                bool user, bool weight, cudaStream_t s) {
  const size_t smem = degrid_smem_bytes(sizeof(real), J, win_rows, win_cols, shape, user, weight);
  ApplyArgs<real> b = a;
  b.win_bytes = int(window_bytes(sizeof(real), win_rows, win_cols, shape, false));
  b.stage_bytes = int(stage_bytes(sizeof(real), J, user, weight));
  return launch_apply<real, true>(true, b, poly, J, ntasks, smem, shape.threads, s);
}
template <typename real>
cudaError_t launch_grid_group(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                              int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                              bool user, bool weight, cudaStream_t s) {
  const size_t smem = grid_smem_bytes(sizeof(real), J, win_rows, win_cols, shape, user, weight);
  ApplyArgs<real> b = a;
  b.win_bytes = int(window_bytes(sizeof(real), win_rows, win_cols, shape, true));
  return launch_apply<real, true>(false, b, poly, J, ntasks, smem, shape.threads, s);
}

template <typename real>
cudaError_t launch_fold_group(const FoldArgs *folds, int nch, int max_tiles, cudaStream_t s) {
  if (nch == 0 || max_tiles == 0) return cudaSuccess;
  fold_group_kernel<real><<<dim3(max_tiles, nch), dim3(32, 8), 0, s>>>(folds);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_pad_group(const ChannelIO<real> *chans, int nch, int64_t max_pixels,
                             cudaStream_t s) {
  if (nch == 0 || max_pixels == 0) return cudaSuccess;
  pad_group_kernel<real><<<dim3(unsigned((max_pixels + 255) / 256), nch), 256, 0, s>>>(chans);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_crop_group(const ChannelIO<real> *chans, int nch, int64_t max_pixels,
                              cudaStream_t s) {
  if (nch == 0 || max_pixels == 0) return cudaSuccess;
  crop_group_kernel<real><<<dim3(unsigned((max_pixels + 255) / 256), nch), 256, 0, s>>>(chans);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_compact_group(const ChannelIO<real> *chans, int nch, int64_t max_vis,
                                 cudaStream_t s) {
  if (nch == 0 || max_vis == 0) return cudaSuccess;
  const int bx = std::max(1, std::min(int((max_vis + 255) / 256), 2048));
  compact_group_kernel<real><<<dim3(bx, nch), 256, 0, s>>>(chans);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_expand_group(const ChannelIO<real> *chans, int nch, int64_t max_slots,
                                cudaStream_t s) {
  if (nch == 0 || max_slots == 0) return cudaSuccess;
  const int bx = std::max(1, std::min(int((max_slots + 255) / 256), 2048));
  expand_group_kernel<real><<<dim3(bx, nch), 256, 0, s>>>(chans);
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
cudaError_t launch_scale_group(const ChannelIO<real> *chans, int nch, int64_t max_pixels,
                               const double *inv, cudaStream_t s) {
  if (nch == 0 || max_pixels == 0) return cudaSuccess;
  const int bx = std::max(1, std::min(int((max_pixels + 255) / 256), 2048));
  scale_group_kernel<real><<<dim3(bx, nch), 256, 0, s>>>(chans, inv);
  return cudaGetLastError();
}

#define PG_INSTANTIATE_GROUP(real)                                                               \
  template cudaError_t launch_degrid_group<real>(const ApplyArgs<real> &, const PolyTable<real> &,  \
                                                 int, int, int, int, const LaunchShape &, bool,    \
                                                 bool, cudaStream_t);                              \
  template cudaError_t launch_grid_group<real>(const ApplyArgs<real> &, const PolyTable<real> &,    \
                                               int, int, int, int, const LaunchShape &, bool,      \
                                               bool, cudaStream_t);                                \
  template cudaError_t launch_fold_group<real>(const FoldArgs *, int, int, cudaStream_t);          \
  template cudaError_t launch_pad_group<real>(const ChannelIO<real> *, int, int64_t, cudaStream_t); \
  template cudaError_t launch_crop_group<real>(const ChannelIO<real> *, int, int64_t,              \
                                               cudaStream_t);                                      \
  template cudaError_t launch_compact_group<real>(const ChannelIO<real> *, int, int64_t,           \
                                                  cudaStream_t);                                   \
  template cudaError_t launch_expand_group<real>(const ChannelIO<real> *, int, int64_t,            \
                                                 cudaStream_t);                                    \
  template cudaError_t launch_sq_norm_group<real>(const ChannelIO<real> *, int, double *, double *, \
                                                  cudaStream_t);                                   \
  template cudaError_t launch_scale_group<real>(const ChannelIO<real> *, int, int64_t,             \
                                                const double *, cudaStream_t);

PG_INSTANTIATE_GROUP(float)
PG_INSTANTIATE_GROUP(double)

}  // namespace pg
