// sm_103a kernels of the measurement operator Phi = G F Z S and its adjoint.
//
// The FFT F is cuFFT; every other stage is here:
//   pad_kernel     Z S     image -> zero-padded grid, correction and scale fused
//   degrid_kernel  G       grid window staged in shared memory, one lane per
//                          work item (a base cell and up to K visibilities),
//                          visibilities in slot order (coalesced per warp)
//   grid_kernel    G^H     lanes accumulate a J x J block per work item in
//                          registers and flush it into a warp-private window
//                          in a fixed order; warp windows are summed in order
//   fold_kernel            fixed-order sum of the task windows covering a cell
//   crop_kernel    S^H Z^H grid -> image, correction and scale fused
//   compact/expand         caller order <-> slot order of the visibilities
// No float atomics are used anywhere, so every result is bit-reproducible for
// a given plan and launch shape.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "device_kernels.h"
#include "gridding_device.cuh"

namespace pg {
namespace {
using namespace dev;

// The permutations are random 8-byte gathers: each thread keeps four of them
// in flight (indices first, then the gathered values), which is what bounds
// them, not instructions.
constexpr int kPermUnroll = 4;
template <typename real>
__global__ void compact_kernel(const cplx<real> *__restrict__ slots,
                               const int32_t *__restrict__ user_slot,
                               cplx<real> *__restrict__ out, int64_t M) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t m0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; m0 < M;
       m0 += kPermUnroll * stride) {
    int32_t src[kPermUnroll];
    cplx<real> v[kPermUnroll];
#pragma unroll
    for (int r = 0; r < kPermUnroll; ++r)
      src[r] = m0 + r * stride < M ? __ldcs(user_slot + m0 + r * stride) : -1;
#pragma unroll
    for (int r = 0; r < kPermUnroll; ++r) v[r] = src[r] >= 0 ? slots[src[r]] : cplx<real>{0, 0};
#pragma unroll
    for (int r = 0; r < kPermUnroll; ++r)
      if (m0 + r * stride < M) __stcs(out + m0 + r * stride, v[r]);
  }
}
// Gathered loads of the caller-ordered visibilities at L2 evict-last
// priority (launch_expand's keep_in): l2_keep_policy / load_keep of
// gridding_device.cuh.
template <typename real>
__global__ void expand_kernel(const cplx<real> *__restrict__ in,
                              const int32_t *__restrict__ slot_user,
                              cplx<real> *__restrict__ slots, int64_t S, bool keep,
                              const cplx<real> *__restrict__ w) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  const unsigned long long pol = l2_keep_policy();
  for (int64_t s0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s0 < S;
       s0 += kPermUnroll * stride) {
    int32_t m[kPermUnroll];
    cplx<real> v[kPermUnroll];
#pragma unroll
    for (int r = 0; r < kPermUnroll; ++r)
      m[r] = s0 + r * stride < S ? __ldcs(slot_user + s0 + r * stride) : -1;
#pragma unroll
    for (int r = 0; r < kPermUnroll; ++r)
      v[r] = m[r] < 0 ? cplx<real>{0, 0} : keep ? load_keep(in + m[r], pol) : in[m[r]];
    if (w) {
      // conj(w) v: G^H holds the conjugated entries of G
#pragma unroll
      for (int r = 0; r < kPermUnroll; ++r)
        if (s0 + r * stride < S) {
          const cplx<real> c = __ldcs(w + s0 + r * stride);
          v[r] = cplx<real>{c.x * v[r].x + c.y * v[r].y, c.x * v[r].y - c.y * v[r].x};
        }
    }
#pragma unroll
    for (int r = 0; r < kPermUnroll; ++r)
      if (s0 + r * stride < S) __stcs(slots + s0 + r * stride, v[r]);
  }
}

template <typename real>
__global__ void fold_kernel(const FoldArgs f) {
  dev::pdl_launch_next();
  dev::pdl_wait();  // the task windows are the previous kernel's output
  fold_tile<real>(f, blockIdx.x);
}

template <typename real>
__global__ void pad_kernel(const cplx<real> *__restrict__ x, const real *__restrict__ su,
                           const real *__restrict__ sv, cplx<real> *__restrict__ grid, int Nx,
                           int Ny, int Nu, int x0, int y0) {
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= int64_t(Nx) * Ny) return;
  const int j = int(idx / Nx), i = int(idx - int64_t(j) * Nx);
  const real s = su[i] * sv[j];
  const cplx<real> v = x[idx];
  grid[int64_t(y0 + j) * Nu + x0 + i] = cplx<real>{s * v.x, s * v.y};
}

template <typename real>
__global__ void crop_kernel(const cplx<real> *__restrict__ grid, const real *__restrict__ su,
                            const real *__restrict__ sv, cplx<real> *__restrict__ x, int Nx,
                            int Ny, int Nu, int x0, int y0) {
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= int64_t(Nx) * Ny) return;
  const int j = int(idx / Nx), i = int(idx - int64_t(j) * Nx);
  const real s = su[i] * sv[j];
  const cplx<real> v = grid[int64_t(y0 + j) * Nu + x0 + i];
  x[idx] = cplx<real>{s * v.x, s * v.y};
}

template <typename real>
__global__ void from_c128_kernel(const double2 *__restrict__ src, cplx<real> *__restrict__ dst,
                                 int64_t n) {
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x) {
    const double2 v = src[k];
    dst[k] = cplx<real>{real(v.x), real(v.y)};
  }
}
template <typename real>
__global__ void to_c128_kernel(const cplx<real> *__restrict__ src, double2 *__restrict__ dst,
                               int64_t n) {
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x) {
    const cplx<real> v = src[k];
    dst[k] = double2{double(v.x), double(v.y)};
  }
}

// Fixed-shape two-stage reduction: block b sums elements b*256+tid + k*stride
// in ascending k, then a fixed tree; the second stage sums the block partials
// in a fixed tree.  The result depends only on n.
template <typename real>
__global__ void sq_norm_partial(const cplx<real> *__restrict__ x, int64_t n,
                                double *__restrict__ partial) {
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
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}
__global__ void sq_norm_final(const double *__restrict__ partial, int n, double *__restrict__ out) {
  __shared__ double red[512];
  red[threadIdx.x] = threadIdx.x < n ? partial[threadIdx.x] : 0.0;
  __syncthreads();
  for (int w = 256; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

template <typename real>
__global__ void scale_kernel(cplx<real> *x, int64_t n, real s) {
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x) {
    cplx<real> v = x[k];
    v.x *= s;
    v.y *= s;
    x[k] = v;
  }
}
template <typename real>
__global__ void fill_kernel(cplx<real> *x, int64_t n, real value) {
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x)
    x[k] = cplx<real>{value, real(0)};
}

// x <- x * real(1 / sqrt(*sq)) (0 when *sq is not positive).
template <typename real>
__global__ void scale_rsqrt_kernel(cplx<real> *x, int64_t n, const double *__restrict__ sq) {
  const double v = sqrt(*sq);
  const real s = v > 0 ? real(1.0 / v) : real(0);
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x) {
    cplx<real> w = x[k];
    w.x *= s;
    w.y *= s;
    x[k] = w;
  }
}

// a <- a * b * scale (complex, element-wise).
template <typename real>
__global__ void cmul_scale_kernel(cplx<real> *__restrict__ a, const cplx<real> *__restrict__ b,
                                  int64_t n, real scale) {
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x) {
    const cplx<real> x = a[k], y = b[k];
    a[k] = cplx<real>{scale * (x.x * y.x - x.y * y.y), scale * (x.x * y.y + x.y * y.x)};
  }
}
// a <- a * b or a * conj(b) (complex, element-wise).
template <typename real, bool CONJ>
__global__ void cmul_kernel(cplx<real> *__restrict__ a, const cplx<real> *__restrict__ b,
                            int64_t n) {
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x) {
    const cplx<real> x = a[k], y = b[k];
    const real yi = CONJ ? -y.y : y.y;
    a[k] = cplx<real>{x.x * y.x - x.y * yi, x.x * yi + x.y * y.x};
  }
}

// x <- 0, x[index] <- 1.
template <typename real>
__global__ void delta_kernel(cplx<real> *x, int64_t n, int64_t index) {
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x)
    x[k] = cplx<real>{k == index ? real(1) : real(0), real(0)};
}

int stream_blocks(int64_t n, int threads) {
  const int64_t b = (n + threads - 1) / threads;
  return int(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

}  // namespace

size_t degrid_smem_bytes(int precision_bytes, int J, int win_rows, int win_cols,
                         const LaunchShape &shape, bool user, int group, int nsub) {
  return window_bytes(precision_bytes, win_rows, win_cols, shape, false, group) + kHeaderBytes +
         size_t(shape.threads / 32) * stage_bytes(precision_bytes, J, user) +
         coefficient_bytes(precision_bytes, J, nsub);
}
size_t grid_smem_bytes(int precision_bytes, int J, int win_rows, int win_cols,
                       const LaunchShape &shape, bool, int group, int nsub) {
  return window_bytes(precision_bytes, win_rows, win_cols, shape, true, group) + kHeaderBytes +
         coefficient_bytes(precision_bytes, J, nsub);
}

template <typename real>
cudaError_t launch_degrid(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                          int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                          cudaStream_t s) {
  const bool user = a.slot_user != nullptr;
  const size_t smem = degrid_smem_bytes(sizeof(real), J, win_rows, win_cols, shape, user,
                                        a.group_cells, poly_nsub(poly));
  ApplyArgs<real> b = a;
  b.win_bytes = int(window_bytes(sizeof(real), win_rows, win_cols, shape, false, a.group_cells));
  b.stage_bytes = int(stage_bytes(sizeof(real), J, user));
  return launch_apply<real, false>(true, b, poly, J, ntasks, smem, shape.threads, s);
}
size_t normal_smem_bytes(int precision_bytes, int J, int win_rows, int win_cols,
                         const LaunchShape &shape, int group, int nsub) {
  if (precision_bytes != 4 || group != 1 || J < 1 || J > 6) return 0;
  return window_bytes(precision_bytes, win_rows, win_cols, shape, false, group) +
         window_bytes(precision_bytes, win_rows, win_cols, shape, true, group) + kHeaderBytes +
         coefficient_bytes(precision_bytes, J, nsub);
}

template <typename real, int J, bool SUB>
cudaError_t launch_normal_one(const ApplyArgs<real> &a, const PolyTable<real> &poly, int ntasks,
                              size_t smem, int threads, cudaStream_t s) {
  auto fn = normal_kernel<real, J, SUB>;
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  return launch_chain(fn, dim3(ntasks), dim3(threads), smem, s, a, poly);
}

template <typename real>
cudaError_t launch_normal(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                          int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                          cudaStream_t s) {
  if constexpr (sizeof(real) != 4) {
    return cudaErrorInvalidValue;
  } else {
    const size_t smem = normal_smem_bytes(sizeof(real), J, win_rows, win_cols, shape,
                                          a.group_cells, poly_nsub(poly));
    if (smem == 0 || a.slot_user || a.group) return cudaErrorInvalidValue;
    if (ntasks == 0) return cudaSuccess;
    ApplyArgs<real> b = a;
    b.stage_bytes = int(window_bytes(sizeof(real), win_rows, win_cols, shape, false, 1));
    b.win_bytes = b.stage_bytes + int(window_bytes(sizeof(real), win_rows, win_cols, shape, true, 1));
    const bool sub = poly.nsub_u > 1 || poly.nsub_v > 1;
    switch (J) {
#define PG_NORMAL(JJ)                                                                        \
  case JJ:                                                                                   \
    return sub ? launch_normal_one<real, JJ, true>(b, poly, ntasks, smem, shape.threads, s)  \
               : launch_normal_one<real, JJ, false>(b, poly, ntasks, smem, shape.threads, s);
      PG_NORMAL(1)
      PG_NORMAL(2)
      PG_NORMAL(3)
      PG_NORMAL(4)
      PG_NORMAL(5)
      PG_NORMAL(6)
#undef PG_NORMAL
    }
    return cudaErrorInvalidValue;
  }
}

template <typename real>
cudaError_t launch_grid(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                        int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                        cudaStream_t s) {
  const bool user = a.slot_user != nullptr;
  const size_t smem = grid_smem_bytes(sizeof(real), J, win_rows, win_cols, shape, user,
                                      a.group_cells, poly_nsub(poly));
  ApplyArgs<real> b = a;
  b.win_bytes = int(window_bytes(sizeof(real), win_rows, win_cols, shape, true, a.group_cells));
  return launch_apply<real, false>(false, b, poly, J, ntasks, smem, shape.threads, s);
}

template <typename real, int J, bool SUB>
cudaError_t launch_walk_one(const WalkArgs<real> &a, const PolyTable<real> &poly, int ntasks,
                            int threads, cudaStream_t s) {
  const size_t smem = walk_smem_bytes(sizeof(real), a.win_rows, a.win_stride, a.max_steps, J,
                                      poly_nsub(poly));
  auto fn = walk_grid_kernel<real, J, SUB>;
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  fn<<<ntasks, threads, smem, s>>>(a, poly);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_walk_grid(const WalkArgs<real> &a, const PolyTable<real> &poly, int J,
                             int ntasks, int threads, cudaStream_t s) {
  if (ntasks == 0) return cudaSuccess;
  if (threads != 32 * kWalkWarps || a.win_stride % 2 == 0 || a.max_steps < 1)
    return cudaErrorInvalidValue;
  const bool sub = poly.nsub_u > 1 || poly.nsub_v > 1;
  switch (J) {
#define PG_WALK(JJ)                                                        \
  case JJ:                                                                 \
    return sub ? launch_walk_one<real, JJ, true>(a, poly, ntasks, threads, s) \
               : launch_walk_one<real, JJ, false>(a, poly, ntasks, threads, s);
    PG_WALK(1)
    PG_WALK(2)
    PG_WALK(3)
    PG_WALK(4)
    PG_WALK(5)
    PG_WALK(6)
    PG_WALK(7)
    PG_WALK(8)
#undef PG_WALK
  }
  return cudaErrorInvalidValue;
}

template <typename real>
cudaError_t launch_fold(const FoldArgs &f, cudaStream_t s) {
  return launch_chain(fold_kernel<real>, dim3(f.ntu * f.ntv), dim3(32, 8), 0, s, f);
}

template <typename real>
cudaError_t launch_pad(const void *x, const real *su, const real *sv, void *grid, int Nx, int Ny,
                       int Nu, int x0, int y0, cudaStream_t s) {
  const int64_t n = int64_t(Nx) * Ny;
  if (n == 0) return cudaSuccess;
  pad_kernel<real><<<int((n + 255) / 256), 256, 0, s>>>(
      static_cast<const cplx<real> *>(x), su, sv, static_cast<cplx<real> *>(grid), Nx, Ny, Nu, x0,
      y0);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_crop(const void *grid, const real *su, const real *sv, void *x, int Nx, int Ny,
                        int Nu, int x0, int y0, cudaStream_t s) {
  const int64_t n = int64_t(Nx) * Ny;
  if (n == 0) return cudaSuccess;
  crop_kernel<real><<<int((n + 255) / 256), 256, 0, s>>>(
      static_cast<const cplx<real> *>(grid), su, sv, static_cast<cplx<real> *>(x), Nx, Ny, Nu,
      x0, y0);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_compact(const void *slots, const int32_t *user_slot, void *out, int64_t M,
                           cudaStream_t s) {
  if (M == 0) return cudaSuccess;
  compact_kernel<real><<<stream_blocks(M, 256), 256, 0, s>>>(
      static_cast<const cplx<real> *>(slots), user_slot, static_cast<cplx<real> *>(out), M);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_expand(const void *in, const int32_t *slot_user, void *slots, int64_t S,
                          cudaStream_t s, bool keep_in, const void *w) {
  if (S == 0) return cudaSuccess;
  expand_kernel<real><<<stream_blocks(S, 256), 256, 0, s>>>(
      static_cast<const cplx<real> *>(in), slot_user, static_cast<cplx<real> *>(slots), S,
      keep_in, static_cast<const cplx<real> *>(w));
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_from_c128(const void *src, void *dst, int64_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  from_c128_kernel<real><<<stream_blocks(n, 256), 256, 0, s>>>(
      static_cast<const double2 *>(src), static_cast<cplx<real> *>(dst), n);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_to_c128(const void *src, void *dst, int64_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  to_c128_kernel<real><<<stream_blocks(n, 256), 256, 0, s>>>(
      static_cast<const cplx<real> *>(src), static_cast<double2 *>(dst), n);
  return cudaGetLastError();
}

template <typename real>
cudaError_t launch_sq_norm(const void *x, int64_t n, double *partial, double *out,
                           cudaStream_t s) {
  sq_norm_partial<real><<<kNormBlocks, 256, 0, s>>>(static_cast<const cplx<real> *>(x), n,
                                                     partial);
  sq_norm_final<<<1, kNormBlocks, 0, s>>>(partial, kNormBlocks, out);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_scale(void *x, int64_t n, double scale, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  scale_kernel<real><<<stream_blocks(n, 256), 256, 0, s>>>(static_cast<cplx<real> *>(x), n,
                                                           real(scale));
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_cmul_scale(void *a, const void *b, int64_t n, double scale, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  cmul_scale_kernel<real><<<stream_blocks(n, 256), 256, 0, s>>>(
      static_cast<cplx<real> *>(a), static_cast<const cplx<real> *>(b), n, real(scale));
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_cmul(void *a, const void *b, int64_t n, bool conj_b, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  auto *pa = static_cast<cplx<real> *>(a);
  auto *pb = static_cast<const cplx<real> *>(b);
  if (conj_b)
    cmul_kernel<real, true><<<stream_blocks(n, 256), 256, 0, s>>>(pa, pb, n);
  else
    cmul_kernel<real, false><<<stream_blocks(n, 256), 256, 0, s>>>(pa, pb, n);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_delta(void *x, int64_t n, int64_t index, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  delta_kernel<real><<<stream_blocks(n, 256), 256, 0, s>>>(static_cast<cplx<real> *>(x), n, index);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_scale_rsqrt(void *x, int64_t n, const double *sq, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  scale_rsqrt_kernel<real><<<stream_blocks(n, 256), 256, 0, s>>>(static_cast<cplx<real> *>(x), n,
                                                                 sq);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_fill(void *x, int64_t n, double value, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  fill_kernel<real><<<stream_blocks(n, 256), 256, 0, s>>>(static_cast<cplx<real> *>(x), n,
                                                          real(value));
  return cudaGetLastError();
}

#define PG_INSTANTIATE(real)                                                                    \
  template cudaError_t launch_degrid<real>(const ApplyArgs<real> &, const PolyTable<real> &, int, \
                                           int, int, int, const LaunchShape &, cudaStream_t);   \
  template cudaError_t launch_grid<real>(const ApplyArgs<real> &, const PolyTable<real> &, int,   \
                                         int, int, int, const LaunchShape &, cudaStream_t);     \
  template cudaError_t launch_normal<real>(const ApplyArgs<real> &, const PolyTable<real> &, int, \
                                           int, int, int, const LaunchShape &, cudaStream_t);   \
  template cudaError_t launch_fold<real>(const FoldArgs &, cudaStream_t);                       \
  template cudaError_t launch_walk_grid<real>(const WalkArgs<real> &, const PolyTable<real> &,  \
                                              int, int, int, cudaStream_t);                     \
  template cudaError_t launch_pad<real>(const void *, const real *, const real *, void *, int,  \
                                        int, int, int, int, cudaStream_t);                      \
  template cudaError_t launch_crop<real>(const void *, const real *, const real *, void *, int, \
                                         int, int, int, int, cudaStream_t);                     \
  template cudaError_t launch_compact<real>(const void *, const int32_t *, void *, int64_t,      \
                                           cudaStream_t);                                      \
  template cudaError_t launch_expand<real>(const void *, const int32_t *, void *, int64_t,       \
                                          cudaStream_t, bool, const void *);                   \
  template cudaError_t launch_from_c128<real>(const void *, void *, int64_t, cudaStream_t);     \
  template cudaError_t launch_to_c128<real>(const void *, void *, int64_t, cudaStream_t);       \
  template cudaError_t launch_sq_norm<real>(const void *, int64_t, double *, double *,          \
                                            cudaStream_t);                                      \
  template cudaError_t launch_scale<real>(void *, int64_t, double, cudaStream_t);               \
  template cudaError_t launch_fill<real>(void *, int64_t, double, cudaStream_t);                 \
  template cudaError_t launch_scale_rsqrt<real>(void *, int64_t, const double *, cudaStream_t);   \
  template cudaError_t launch_cmul_scale<real>(void *, const void *, int64_t, double, cudaStream_t); \
  template cudaError_t launch_delta<real>(void *, int64_t, int64_t, cudaStream_t);              \
  template cudaError_t launch_cmul<real>(void *, const void *, int64_t, bool, cudaStream_t);

PG_INSTANTIATE(float)
PG_INSTANTIATE(double)

}  // namespace pg
