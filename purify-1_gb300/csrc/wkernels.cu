// sm_103a kernels of the w-projection gridding operator (G and G^H with one
// kernel row per visibility).  Row m's S x S taps are rebuilt on the fly from
// its stored rank-3 factors, K = A_0 B_0^T + A_1 B_1^T + A_2 B_2^T
// (wplan.h), over the row's nonzero terms only (rank 1 to 3, from the row
// code).  One warp handles one visibility at a time; lane l covers row
// r = l / S of each group of R = 32 / S rows and column c = l % S, two row
// groups per step.
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

__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_one() {
  asm volatile("cp.async.wait_group 1;\n" ::: "memory");
}

// Per-warp software pipeline over the visibilities i = first, first + nw, ...
// of a task: while visibility i is computed, the row factors of the next one
// are on their way into the other half of the warp's factor buffer
// (cp.async), and the code, factor offset, weight and visibility of the one
// after that are being loaded into registers.
// Stored factor terms of a row: the popcount of the code's term mask.
__device__ __forceinline__ int row_rank(int code) { return __popc((code >> 24) & 7); }

// Tap (row j, the lane's column) of a row: sum over the stored terms of
// A_e[j] b[e], with b[e] = B_e[column] held by the lane.  The rank is the same
// for the whole warp (one visibility).
template <typename C>
__device__ __forceinline__ C row_tap(const C *fbuf, int S, int rank, int j, const C (&b)[3]) {
  C k = cmul(fbuf[j], b[0]);
  if (rank > 1) cfma(k, fbuf[S + j], b[1]);
  if (rank > 2) cfma(k, fbuf[2 * S + j], b[2]);
  return k;
}
template <typename C>
__device__ __forceinline__ void column_factors(const C *fbuf, int S, int rank, int c, bool active,
                                               C (&b)[3]) {
  b[0] = b[1] = b[2] = C{0, 0};
  if (!active) return;
  b[0] = fbuf[rank * S + c];
  if (rank > 1) b[1] = fbuf[(rank + 1) * S + c];
  if (rank > 2) b[2] = fbuf[(rank + 2) * S + c];
}

template <typename real>
struct WPipe {
  using C = cplx<real>;
  const WArgs<real> &a;
  C *fb;  // [2][6 * Smax]
  int lane, nw, end;
  int code1 = 0, code2 = 0;
  int64_t off1 = 0, off2 = 0;
  C w1{0, 0}, w2{0, 0}, y1{0, 0}, y2{0, 0};
  __device__ WPipe(const WArgs<real> &args, C *buf, int l, int n, int e)
      : a(args), fb(buf), lane(l), nw(n), end(e) {}
  __device__ __forceinline__ void meta(int i, int &code, int64_t &off, C &w, C &y, bool vis_in) {
    if (i < end) {
      code = a.code[i];
      off = a.factor[i];
      w = static_cast<const C *>(a.weight)[i];
      if (vis_in) y = static_cast<const C *>(a.slot_in)[i];
    }
  }
  __device__ __forceinline__ void issue(int i, int code, int64_t off, int buf) {
    if (i < end) {
      const int n = 2 * row_rank(code) * ((code >> 16) & 0xff);
      const C *src = static_cast<const C *>(a.factors) + off;
      C *dst = fb + buf * 6 * a.Smax;
      for (int k = lane; k < n; k += 32) cp_async<sizeof(C)>(dst + k, src + k);
    }
    cp_async_commit();
  }
};

template <typename real>
__global__ void __launch_bounds__(128) wdegrid_kernel(const WArgs<real> a) {
  using C = cplx<real>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int task_id = a.order ? a.order[blockIdx.x] : int(blockIdx.x);
  const Task tk = a.tasks[task_id];
  const int WW = tk.W + a.Smax - 1, WH = tk.H + a.Smax - 1;
  C *win = reinterpret_cast<C *>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  C *fb = reinterpret_cast<C *>(smem_raw + a.win_bytes) + warp * 2 * 6 * a.Smax;
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
  C *out = static_cast<C *>(a.slot_out);
  const int first = tk.batch_begin + warp;
  WPipe<real> pp(a, fb, lane, nw, tk.batch_end);
  int code0 = 0;
  int64_t off0 = 0;
  C w0{0, 0}, y0{0, 0};
  pp.meta(first, code0, off0, w0, y0, false);
  pp.meta(first + nw, pp.code1, pp.off1, pp.w1, pp.y1, false);
  pp.issue(first, code0, off0, 0);
  int buf = 0;
  for (int i = first; i < tk.batch_end; i += nw) {
    pp.issue(i + nw, pp.code1, pp.off1, buf ^ 1);
    pp.meta(i + 2 * nw, pp.code2, pp.off2, pp.w2, pp.y2, false);
    cp_async_wait_one();
    __syncwarp();  // every lane's factor copies for visibility i have landed
    const C *fbuf = fb + buf * 6 * a.Smax;
    const int lp = code0 & 0xff, lq = (code0 >> 8) & 0xff, S = (code0 >> 16) & 0xff;
    const int rank = row_rank(code0);
    const int R = 32 / S, r = lane / S, c = lane - r * S;
    const bool active = r < R;
    C b[3];
    column_factors(fbuf, S, rank, c, active, b);
    C acc{0, 0}, acc2{0, 0};
    for (int jv0 = 0; jv0 < S; jv0 += 2 * R) {
      const int ja = jv0 + r, jb = jv0 + R + r;
      if (active && ja < S) cfma(acc, row_tap(fbuf, S, rank, ja, b), win[(lp + ja) * WW + lq + c]);
      if (active && jb < S) cfma(acc2, row_tap(fbuf, S, rank, jb, b), win[(lp + jb) * WW + lq + c]);
    }
    acc.x += acc2.x;
    acc.y += acc2.y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    if (lane == 0) out[i] = cmul(acc, w0);
    __syncwarp();  // this half of the factor buffer is refilled two visibilities on
    code0 = pp.code1;
    off0 = pp.off1;
    w0 = pp.w1;
    pp.code1 = pp.code2;
    pp.off1 = pp.off2;
    pp.w1 = pp.w2;
    buf ^= 1;
  }
  cp_async_wait_all();
}

template <typename real>
__global__ void __launch_bounds__(128) wgrid_kernel(const WArgs<real> a) {
  using C = cplx<real>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int task_id = a.order ? a.order[blockIdx.x] : int(blockIdx.x);
  const Task tk = a.tasks[task_id];
  const int WW = tk.W + a.Smax - 1, WH = tk.H + a.Smax - 1, WN = WW * WH;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  C *wins = reinterpret_cast<C *>(smem_raw);
  C *fb = reinterpret_cast<C *>(smem_raw + a.win_bytes) + warp * 2 * 6 * a.Smax;
  for (int idx = threadIdx.x; idx < nw * WN; idx += blockDim.x) wins[idx] = C{0, 0};
  __syncthreads();
  C *mine = wins + warp * WN;
  const int first = tk.batch_begin + warp;
  WPipe<real> pp(a, fb, lane, nw, tk.batch_end);
  int code0 = 0;
  int64_t off0 = 0;
  C w0{0, 0}, y0{0, 0};
  pp.meta(first, code0, off0, w0, y0, true);
  pp.meta(first + nw, pp.code1, pp.off1, pp.w1, pp.y1, true);
  pp.issue(first, code0, off0, 0);
  int buf = 0;
  for (int i = first; i < tk.batch_end; i += nw) {
    pp.issue(i + nw, pp.code1, pp.off1, buf ^ 1);
    pp.meta(i + 2 * nw, pp.code2, pp.off2, pp.w2, pp.y2, true);
    cp_async_wait_one();
    __syncwarp();  // every lane's factor copies for visibility i have landed
    const C *fbuf = fb + buf * 6 * a.Smax;
    const int lp = code0 & 0xff, lq = (code0 >> 8) & 0xff, S = (code0 >> 16) & 0xff;
    const int rank = row_rank(code0);
    // conj(weight) * y: G^H holds the conjugated entries of G
    const C z{w0.x * y0.x + w0.y * y0.y, w0.x * y0.y - w0.y * y0.x};
    const int R = 32 / S, r = lane / S, c = lane - r * S;
    const bool active = r < R;
    C b[3];
    column_factors(fbuf, S, rank, c, active, b);
    // All S^2 cells of one visibility are distinct, so the lanes never touch
    // the same cell within it, and the two rows a lane updates per step are
    // different cells; visibilities are ordered by __syncwarp.
    for (int jv0 = 0; jv0 < S; jv0 += 2 * R) {
      const int ja = jv0 + r, jb = jv0 + R + r;
      const bool oka = active && ja < S, okb = active && jb < S;
      C ka{0, 0}, kb{0, 0}, va{0, 0}, vb{0, 0};
      C *ca = mine + (lp + ja) * WW + lq + c;
      C *cb = mine + (lp + jb) * WW + lq + c;
      if (oka) {
        ka = row_tap(fbuf, S, rank, ja, b);
        va = *ca;
      }
      if (okb) {
        kb = row_tap(fbuf, S, rank, jb, b);
        vb = *cb;
      }
      // conj(K) z
      if (oka) {
        va.x = fma(ka.x, z.x, fma(ka.y, z.y, va.x));
        va.y = fma(ka.x, z.y, fma(-ka.y, z.x, va.y));
        *ca = va;
      }
      if (okb) {
        vb.x = fma(kb.x, z.x, fma(kb.y, z.y, vb.x));
        vb.y = fma(kb.x, z.y, fma(-kb.y, z.x, vb.y));
        *cb = vb;
      }
    }
    __syncwarp();
    code0 = pp.code1;
    off0 = pp.off1;
    w0 = pp.w1;
    y0 = pp.y1;
    pp.code1 = pp.code2;
    pp.off1 = pp.off2;
    pp.w1 = pp.w2;
    pp.y1 = pp.y2;
    buf ^= 1;
  }
  cp_async_wait_all();
  __syncthreads();
  C *out = static_cast<C *>(a.tilebuf) + size_t(task_id) * a.slot_stride;
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
         size_t(threads / 32) * 2 * 6 * Smax * 2 * sizeof(real);
}
template <typename real>
size_t wgrid_smem_bytes(int win_rows, int win_cols, int Smax, int threads) {
  return wwindow_bytes(sizeof(real), win_rows, win_cols, threads, true) +
         size_t(threads / 32) * 2 * 6 * Smax * 2 * sizeof(real);
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
