// sm_103a kernels of the w-projection gridding operator (G and G^H with one
// kernel row per visibility).  Row m's S x S taps are rebuilt on the fly from
// its stored rank-3 factors, K = A_0 B_0^T + A_1 B_1^T + A_2 B_2^T
// (wplan.h).  One warp handles one visibility at a time; lane l covers row
// r = l / S of each group of R = 32 / S rows and column c = l % S.
#include <cuda_runtime.h>

#include <cstdint>

#include "wkernels.h"

namespace pg {
namespace {

template <typename real>
struct Cplx;
template <>
struct Cplx<float> {
  using type = float2;
};
template <>
struct Cplx<double> {
  using type = double2;
};
template <typename real>
using cplx = typename Cplx<real>::type;

template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
  return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename C>
__device__ __forceinline__ void cfma(C &acc, C a, C b) {
  acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}

template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(BYTES)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Stages the 6 S factors of a row into the warp's buffer.
template <typename C>
__device__ __forceinline__ void stage_factors(const C *src, C *buf, int S, int lane) {
  for (int k = lane; k < 6 * S; k += 32) buf[k] = src[k];
  __syncwarp();
}

template <typename real>
__global__ void __launch_bounds__(128) wdegrid_kernel(const WArgs<real> a) {
  using C = cplx<real>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Task tk = a.tasks[blockIdx.x];
  const int WW = tk.W + a.Smax - 1, WH = tk.H + a.Smax - 1;
  C *win = reinterpret_cast<C *>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  C *fbuf = reinterpret_cast<C *>(smem_raw + a.win_bytes) + warp * 6 * a.Smax;
  const C *grid = static_cast<const C *>(a.grid);
  for (int idx = threadIdx.x; idx < WW * WH; idx += blockDim.x) {
    const int lp = idx / WW, lq = idx - lp * WW;
    int p = tk.P + lp;
    if (p >= a.Nv) p -= a.Nv;
    int q = tk.Q + lq;
    if (q >= a.Nu) q -= a.Nu;
    cp_async<sizeof(C)>(win + idx, grid + size_t(p) * a.Nu + q);
  }
  cp_async_wait_all();
  __syncthreads();
  const C *factors = static_cast<const C *>(a.factors);
  const C *weight = static_cast<const C *>(a.weight);
  C *out = static_cast<C *>(a.slot_out);
  for (int i = tk.batch_begin + warp; i < tk.batch_end; i += nw) {
    const int code = a.code[i];
    const int lp = code & 0xff, lq = (code >> 8) & 0xff, S = (code >> 16) & 0xff;
    stage_factors(factors + a.factor[i], fbuf, S, lane);
    const int R = 32 / S, r = lane / S, c = lane - r * S;
    const bool active = r < R;
    C b0{0, 0}, b1{0, 0}, b2{0, 0};
    if (active) {
      b0 = fbuf[3 * S + c];
      b1 = fbuf[4 * S + c];
      b2 = fbuf[5 * S + c];
    }
    C acc{0, 0};
    for (int jv0 = 0; jv0 < S; jv0 += R) {
      const int jv = jv0 + r;
      if (active && jv < S) {
        C k = cmul(fbuf[jv], b0);
        cfma(k, fbuf[S + jv], b1);
        cfma(k, fbuf[2 * S + jv], b2);
        cfma(acc, k, win[(lp + jv) * WW + lq + c]);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    if (lane == 0) out[i] = cmul(acc, weight[i]);
    __syncwarp();  // fbuf is reused by the next visibility
  }
}

template <typename real>
__global__ void __launch_bounds__(128) wgrid_kernel(const WArgs<real> a) {
  using C = cplx<real>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Task tk = a.tasks[blockIdx.x];
  const int WW = tk.W + a.Smax - 1, WH = tk.H + a.Smax - 1, WN = WW * WH;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  C *wins = reinterpret_cast<C *>(smem_raw);
  C *fbuf = reinterpret_cast<C *>(smem_raw + a.win_bytes) + warp * 6 * a.Smax;
  for (int idx = threadIdx.x; idx < nw * WN; idx += blockDim.x) wins[idx] = C{0, 0};
  __syncthreads();
  C *mine = wins + warp * WN;
  const C *factors = static_cast<const C *>(a.factors);
  const C *weight = static_cast<const C *>(a.weight);
  const C *vin = static_cast<const C *>(a.slot_in);
  for (int i = tk.batch_begin + warp; i < tk.batch_end; i += nw) {
    const int code = a.code[i];
    const int lp = code & 0xff, lq = (code >> 8) & 0xff, S = (code >> 16) & 0xff;
    stage_factors(factors + a.factor[i], fbuf, S, lane);
    // conj(weight) * y: G^H holds the conjugated entries of G
    const C w = weight[i], y = vin[i];
    const C z{w.x * y.x + w.y * y.y, w.x * y.y - w.y * y.x};
    const int R = 32 / S, r = lane / S, c = lane - r * S;
    const bool active = r < R;
    C b0{0, 0}, b1{0, 0}, b2{0, 0};
    if (active) {
      b0 = fbuf[3 * S + c];
      b1 = fbuf[4 * S + c];
      b2 = fbuf[5 * S + c];
    }
    // All S^2 cells of one visibility are distinct, so the lanes never touch
    // the same cell within it; visibilities are ordered by __syncwarp.
    for (int jv0 = 0; jv0 < S; jv0 += R) {
      const int jv = jv0 + r;
      if (active && jv < S) {
        C k = cmul(fbuf[jv], b0);
        cfma(k, fbuf[S + jv], b1);
        cfma(k, fbuf[2 * S + jv], b2);
        // conj(K) z
        C *cell = mine + (lp + jv) * WW + lq + c;
        C v = *cell;
        v.x = fma(k.x, z.x, fma(k.y, z.y, v.x));
        v.y = fma(k.x, z.y, fma(-k.y, z.x, v.y));
        *cell = v;
      }
    }
    __syncwarp();
  }
  __syncthreads();
  C *out = static_cast<C *>(a.tilebuf) + size_t(blockIdx.x) * a.slot_stride;
  for (int idx = threadIdx.x; idx < WN; idx += blockDim.x) {
    C s = wins[idx];
    for (int w2 = 1; w2 < nw; ++w2) {
      const C o = wins[w2 * WN + idx];
      s.x += o.x;
      s.y += o.y;
    }
    out[idx] = s;
  }
}

size_t wwindow_bytes(int bytes_real, int win_rows, int win_cols, int threads, bool per_warp) {
  const size_t one = size_t(win_rows) * win_cols * 2 * bytes_real;
  const size_t b = per_warp ? one * size_t(threads / 32) : one;
  return (b + 15) / 16 * 16;
}

}  // namespace

template <typename real>
size_t wdegrid_smem_bytes(int win_rows, int win_cols, int Smax, int threads) {
  return wwindow_bytes(sizeof(real), win_rows, win_cols, threads, false) +
         size_t(threads / 32) * 6 * Smax * 2 * sizeof(real);
}
template <typename real>
size_t wgrid_smem_bytes(int win_rows, int win_cols, int Smax, int threads) {
  return wwindow_bytes(sizeof(real), win_rows, win_cols, threads, true) +
         size_t(threads / 32) * 6 * Smax * 2 * sizeof(real);
}

template <typename real>
cudaError_t launch_wdegrid(const WArgs<real> &a0, int ntasks, int win_rows, int win_cols,
                           int threads, cudaStream_t s) {
  if (ntasks == 0) return cudaSuccess;
  WArgs<real> a = a0;
  a.win_bytes = int(wwindow_bytes(sizeof(real), win_rows, win_cols, threads, false));
  const size_t smem = wdegrid_smem_bytes<real>(win_rows, win_cols, a.Smax, threads);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(
        wdegrid_kernel<real>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  wdegrid_kernel<real><<<ntasks, threads, smem, s>>>(a);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_wgrid(const WArgs<real> &a0, int ntasks, int win_rows, int win_cols,
                         int threads, cudaStream_t s) {
  if (ntasks == 0) return cudaSuccess;
  WArgs<real> a = a0;
  a.win_bytes = int(wwindow_bytes(sizeof(real), win_rows, win_cols, threads, true));
  const size_t smem = wgrid_smem_bytes<real>(win_rows, win_cols, a.Smax, threads);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(
        wgrid_kernel<real>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  wgrid_kernel<real><<<ntasks, threads, smem, s>>>(a);
  return cudaGetLastError();
}

template size_t wdegrid_smem_bytes<float>(int, int, int, int);
template size_t wdegrid_smem_bytes<double>(int, int, int, int);
template size_t wgrid_smem_bytes<float>(int, int, int, int);
template size_t wgrid_smem_bytes<double>(int, int, int, int);
template cudaError_t launch_wdegrid<float>(const WArgs<float> &, int, int, int, int, cudaStream_t);
template cudaError_t launch_wdegrid<double>(const WArgs<double> &, int, int, int, int, cudaStream_t);
template cudaError_t launch_wgrid<float>(const WArgs<float> &, int, int, int, int, cudaStream_t);
template cudaError_t launch_wgrid<double>(const WArgs<double> &, int, int, int, int, cudaStream_t);

}  // namespace pg
