// sm_103a kernels of the w-projection gridding operator (G and G^H with one
// kernel row per visibility).  Row m's S x S taps come from its stored
// factors, K = sum_e A_e B_e^T over the row's nonzero terms (rank 1 to 3,
// from the row code; wplan.h).  Within a visibility, lane l covers row slot
// r = l / S of R = 32 / S and column c = l % S.
#include <cuda_runtime.h>

#include <cstdint>

#include "cplx_ops.cuh"
#include "wkernels.h"

namespace pg {
namespace {

using dev::cplx;
using dev::fma2;
using dev::splat;

// ceil(2^16 / S): for lanes l < 32 and S <= 32, (l m) >> 16 = l / S and
// (32 m) >> 16 = 32 / S exactly (the rounding error is below 1/2048, the
// distance to the next integer at least 1/32).
#define PG_MAGIC(S) ((65535 + (S)) / (S))
__constant__ int kLaneMagic[33] = {
    0,            PG_MAGIC(1),  PG_MAGIC(2),  PG_MAGIC(3),  PG_MAGIC(4),  PG_MAGIC(5),
    PG_MAGIC(6),  PG_MAGIC(7),  PG_MAGIC(8),  PG_MAGIC(9),  PG_MAGIC(10), PG_MAGIC(11),
    PG_MAGIC(12), PG_MAGIC(13), PG_MAGIC(14), PG_MAGIC(15), PG_MAGIC(16), PG_MAGIC(17),
    PG_MAGIC(18), PG_MAGIC(19), PG_MAGIC(20), PG_MAGIC(21), PG_MAGIC(22), PG_MAGIC(23),
    PG_MAGIC(24), PG_MAGIC(25), PG_MAGIC(26), PG_MAGIC(27), PG_MAGIC(28), PG_MAGIC(29),
    PG_MAGIC(30), PG_MAGIC(31), PG_MAGIC(32)};
#undef PG_MAGIC

template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
  return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename C>
__device__ __forceinline__ void cfma(C &acc, C a, C b) {
  acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}

// conj(a) b, and acc += conj(a) b
template <typename C>
__device__ __forceinline__ C cmul_conj(C a, C b) {
  return C{a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x};
}
template <typename C>
__device__ __forceinline__ void cfma_conj(C &acc, C a, C b) {
  acc.x = fma(a.x, b.x, fma(a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(-a.y, b.x, acc.y));
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

// Stored factor terms of a row: the popcount of the code's term mask.
__device__ __forceinline__ int row_rank(int code) { return __popc((code >> 24) & 7); }


// G^H of the w-projection rows with one window per CTA.  The window's rows
// are cut into kBandWarps contiguous bands, one per warp, and every warp walks
// the task's visibilities in plan order, updating only the rows of its band
// (a visibility whose rows miss the band costs the warp a comparison): each
// cell has one writer, which adds the visibilities in plan order.  The rows' factors, codes, weights and visibilities are staged
// in shared memory one chunk (WChunk) at a time, the next chunk's copies in
// flight (cp.async) while the current one is gridded.
constexpr int kBandWarps = 8;

template <typename real>
struct BandStage {
  using C = cplx<real>;
  C *f;         // factor values [chunk_values + 2], from the chunk's aligned start
  int64_t *fo;  // factor offsets [kWChunkVis]
  int *rel;     // factor offsets relative to the staged start [kWChunkVis]
  int *code;    // [kWChunkVis]
  C *w, *y;     // weights (G^H: conj(weight) y after the prep pass), visibilities
};

template <typename real>
__host__ __device__ inline size_t band_stage_bytes(int chunk_values) {
  const size_t c = 2 * sizeof(real);
  auto up = [](size_t b) { return (b + 15) / 16 * 16; };
  return up(c * (chunk_values + 2)) + up(8 * kWChunkVis) + 2 * up(4 * kWChunkVis) +
         2 * up(c * kWChunkVis);
}

template <typename real>
__device__ __forceinline__ BandStage<real> band_stage(unsigned char *base, int chunk_values) {
  using C = cplx<real>;
  auto up = [](size_t b) { return (b + 15) / 16 * 16; };
  BandStage<real> st;
  st.f = reinterpret_cast<C *>(base);
  base += up(sizeof(C) * (chunk_values + 2));
  st.fo = reinterpret_cast<int64_t *>(base);
  base += up(8 * kWChunkVis);
  st.rel = reinterpret_cast<int *>(base);
  base += up(4 * kWChunkVis);
  st.code = reinterpret_cast<int *>(base);
  base += up(4 * kWChunkVis);
  st.w = reinterpret_cast<C *>(base);
  base += up(sizeof(C) * kWChunkVis);
  st.y = reinterpret_cast<C *>(base);
  return st;
}

// First factor value a chunk's staging copies start at: the chunk's first
// value rounded down to a 16-byte boundary.
template <typename real>
__device__ __forceinline__ int64_t band_base(const WChunk &c) {
  return sizeof(real) == 4 ? (c.fbegin & ~int64_t(1)) : c.fbegin;
}

template <typename real, bool VIS>
__device__ __forceinline__ void band_issue(const WArgs<real> &a, const WChunk &c,
                                           const BandStage<real> &st) {
  using C = cplx<real>;
  const int tid = threadIdx.x, nt = blockDim.x;
  // factors in 16-byte pieces over [base, fend rounded up): the factor
  // buffer is allocated with a 16-byte tail, so the last piece stays inside
  const int64_t f0 = band_base<real>(c);
  const int64_t nbytes = (c.fend - f0) * int64_t(sizeof(C));
  const int pieces = int((nbytes + 15) / 16);
  const char *src = reinterpret_cast<const char *>(static_cast<const C *>(a.factors) + f0);
  char *dst = reinterpret_cast<char *>(st.f);
  for (int k = tid; k < pieces; k += nt) cp_async<16>(dst + 16 * k, src + 16 * k);
  const int nv = c.vis_end - c.vis_begin;
  for (int k = tid; k < nv; k += nt) {
    const int i = c.vis_begin + k;
    cp_async<8>(st.fo + k, a.factor + i);
    cp_async<4>(st.code + k, a.code + i);
    cp_async<sizeof(C)>(st.w + k, static_cast<const C *>(a.weight) + i);
    if (VIS) cp_async<sizeof(C)>(st.y + k, static_cast<const C *>(a.slot_in) + i);
  }
  cp_async_commit();
}

// Lane layout of a row of support S: R = 32 / S row slots of S columns, lane
// l at row slot r = l / S, column c = l % S.
__device__ __forceinline__ void lane_layout(int S, int lane, int &R, int &r, int &c) {
  const int m = kLaneMagic[S];
  R = (32 * m) >> 16;
  r = (lane * m) >> 16;
  c = lane - r * S;
}

// Packed complex products.  With P = sum g.x A and Q = sum g.y A over taps,
// sum A g = P + i Q; conj(A) b = A.x b + A.y (b.y, -b.x).
template <typename C>
__device__ __forceinline__ C plus_i(C p, C q) {
  return C{p.x - q.y, p.y + q.x};
}

// G of the w-projection rows: the task's grid window is staged once per CTA,
// the rows' factors, codes and weights one chunk at a time (the next chunk
// in flight while the current one is used), and each warp takes whole
// visibilities of the chunk in turn.  For visibility m, lane (r, c) sums
// A_e[jv] g[jv][c] over its rows jv for each stored term e, then applies
// B_e[c]; a butterfly over the warp adds the lanes.
template <typename real>
__global__ void __launch_bounds__(kBandWarps * 32, 4) wdegrid_band_kernel(const WArgs<real> a) {
  using C = cplx<real>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int task_id = a.order ? a.order[blockIdx.x] : int(blockIdx.x);
  const Task tk = a.tasks[task_id];
  const int WW = tk.W + a.Smax - 1, WH = tk.H + a.Smax - 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  C *win = reinterpret_cast<C *>(smem_raw);
  const size_t sb = band_stage_bytes<real>(a.chunk_values);
  auto stage = [&](int buf) {
    return band_stage<real>(smem_raw + a.win_bytes + buf * sb, a.chunk_values);
  };
  const C *grid = static_cast<const C *>(a.grid);
  for (int idx = threadIdx.x; idx < WW * WH; idx += blockDim.x) {
    const int lp = idx / WW, lq = idx - lp * WW;
    int p = tk.P + lp;
    if (p >= a.Nv) p -= a.Nv;
    int q = tk.Q + lq;
    if (q >= a.Nu) q -= a.Nu;
    cp_async<sizeof(C)>(win + idx, grid + size_t(p) * a.Nu + q);
  }
  cp_async_commit();  // the window travels with the first chunk's group
  C *out = static_cast<C *>(a.slot_out);
  const int c0 = a.task_chunk[task_id], c1 = a.task_chunk[task_id + 1];
  if (c0 < c1) band_issue<real, false>(a, a.chunks[c0], stage(0));
  for (int ch = c0; ch < c1; ++ch) {
    const int buf = (ch - c0) & 1;
    if (ch + 1 < c1)
      band_issue<real, false>(a, a.chunks[ch + 1], stage(buf ^ 1));
    else
      cp_async_commit();
    cp_async_wait_one();
    __syncthreads();
    const WChunk cr = a.chunks[ch];
    const BandStage<real> sg = stage(buf);
    const int64_t f0 = band_base<real>(cr);
    const int nv = cr.vis_end - cr.vis_begin;
    for (int v = warp; v < nv; v += kBandWarps) {
      const int code = sg.code[v];
      const int lp = code & 0xff, lq = (code >> 8) & 0xff, S = (code >> 16) & 0xff;
      const int rank = row_rank(code);
      const C *fr = sg.f + (sg.fo[v] - f0);
      int R, r, c;
      lane_layout(S, lane, R, r, c);
      C y{0, 0};
      if (r < R) {
        const C *g = win + (lp + r) * WW + lq + c;
        const int gs = R * WW;
        if (rank == 1) {
          C p{0, 0}, q{0, 0};
#pragma unroll 2
          for (int jv = r; jv < S; jv += R, g += gs) {
            const C gv = *g, A = fr[jv];
            p = fma2(splat(gv.x), A, p);
            q = fma2(splat(gv.y), A, q);
          }
          y = cmul(fr[S + c], plus_i(p, q));
        } else {
          C s0{0, 0}, s1{0, 0}, s2{0, 0};
          for (int jv = r; jv < S; jv += R, g += gs) {
            const C gv = *g;
            cfma(s0, fr[jv], gv);
            cfma(s1, fr[S + jv], gv);
            if (rank > 2) cfma(s2, fr[2 * S + jv], gv);
          }
          y = cmul(fr[rank * S + c], s0);
          cfma(y, fr[(rank + 1) * S + c], s1);
          if (rank > 2) cfma(y, fr[(rank + 2) * S + c], s2);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        y.x += __shfl_xor_sync(0xffffffffu, y.x, o);
        y.y += __shfl_xor_sync(0xffffffffu, y.y, o);
      }
      if (lane == 0) out[cr.vis_begin + v] = cmul(y, sg.w[v]);
    }
    __syncthreads();  // every warp is done with this buffer before it is refilled
  }
  cp_async_wait_all();
}

template <typename real>
__global__ void __launch_bounds__(kBandWarps * 32, 4) wgrid_band_kernel(const WArgs<real> a) {
  using C = cplx<real>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int task_id = a.order ? a.order[blockIdx.x] : int(blockIdx.x);
  const Task tk = a.tasks[task_id];
  const int WW = tk.W + a.Smax - 1, WH = tk.H + a.Smax - 1, WN = WW * WH;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this warp's band of window rows
  const int band_h = (WH + kBandWarps - 1) / kBandWarps;
  const int band0 = min(warp * band_h, WH), band1 = min(band0 + band_h, WH);
  C *win = reinterpret_cast<C *>(smem_raw);
  const size_t sb = band_stage_bytes<real>(a.chunk_values);
  auto stage = [&](int buf) {
    return band_stage<real>(smem_raw + a.win_bytes + buf * sb, a.chunk_values);
  };
  for (int idx = threadIdx.x; idx < WN; idx += blockDim.x) win[idx] = C{0, 0};
  const int c0 = a.task_chunk[task_id], c1 = a.task_chunk[task_id + 1];
  if (c0 < c1) band_issue<real, true>(a, a.chunks[c0], stage(0));
  for (int ch = c0; ch < c1; ++ch) {
    const int buf = (ch - c0) & 1;
    if (ch + 1 < c1)
      band_issue<real, true>(a, a.chunks[ch + 1], stage(buf ^ 1));
    else
      cp_async_commit();  // empty group: "all but the newest" still means this chunk
    cp_async_wait_one();
    __syncthreads();  // the chunk's copies (and the zeroed window) are visible
    const WChunk cr = a.chunks[ch];
    const BandStage<real> sg = stage(buf);
    const int nv = cr.vis_end - cr.vis_begin;
    // prep, one warp per visibility: the staged factor offset, and the column
    // factors replaced in place by conj(B_e[c]) z with z = conj(weight) y
    // (G^H holds the conjugated entries of G), so
    // conj(K[jv][c]) z = sum_e conj(A_e[jv]) B'_e[c]
    for (int v = warp; v < nv; v += kBandWarps) {
      const int code = sg.code[v], S = (code >> 16) & 0xff, rank = row_rank(code);
      const int rel = int(sg.fo[v] - band_base<real>(cr));
      const C z = cmul_conj(sg.w[v], sg.y[v]);
      C *B = sg.f + rel + rank * S;
      for (int k = lane; k < rank * S; k += 32) B[k] = cmul_conj(B[k], z);
      if (lane == 0) sg.rel[v] = rel;
    }
    __syncthreads();
    for (int v = 0; v < nv; ++v) {
      const int code = sg.code[v];
      const int lp = code & 0xff, S = (code >> 16) & 0xff;
      // the rows of the visibility inside this warp's band
      const int lo = max(lp, band0), hi = min(lp + S, band1);
      if (lo < hi) {
        const int lq = (code >> 8) & 0xff, rank = row_rank(code);
        const C *fr = sg.f + sg.rel[v];
        const int jv0 = lo - lp, nrows = hi - lo;
        int R, r, c;
        lane_layout(S, lane, R, r, c);
        if (r < R) {
          C *cell = win + (lo + r) * WW + lq + c;
          const int cs = R * WW;
          const C *A = fr + jv0;
          if (rank == 1) {
            const C bz = fr[S + c], bzr{bz.y, -bz.x};
            for (int t = r; t < nrows; t += R, cell += cs) {
              const C Av = A[t];
              *cell = fma2(splat(Av.y), bzr, fma2(splat(Av.x), bz, *cell));
            }
          } else {
            const C b0 = fr[rank * S + c], b1 = fr[(rank + 1) * S + c];
            const C b2 = rank > 2 ? fr[(rank + 2) * S + c] : C{0, 0};
            for (int t = r; t < nrows; t += R, cell += cs) {
              const int j = t;
              C cv = *cell;
              cfma_conj(cv, A[j], b0);
              cfma_conj(cv, A[S + j], b1);
              if (rank > 2) cfma_conj(cv, A[2 * S + j], b2);
              *cell = cv;
            }
          }
        }
      }
      __syncwarp();  // this warp's cells of visibility v are written before v + 1
    }
    __syncthreads();  // every warp is done with this buffer before it is refilled
  }
  cp_async_wait_all();
  __syncthreads();
  C *out = static_cast<C *>(a.tilebuf) + size_t(task_id) * a.slot_stride;
  for (int idx = threadIdx.x; idx < WN; idx += blockDim.x) out[idx] = win[idx];
}

// One task window (win_rows x win_cols complex), rounded to 16 bytes.
size_t wwindow_bytes(int bytes_real, int win_rows, int win_cols) {
  const size_t b = size_t(win_rows) * win_cols * 2 * bytes_real;
  return (b + 15) / 16 * 16;
}

}  // namespace

template <typename real>
size_t wdegrid_smem_bytes(int win_rows, int win_cols, int chunk_values) {
  return wwindow_bytes(sizeof(real), win_rows, win_cols) + 2 * band_stage_bytes<real>(chunk_values);
}
template <typename real>
size_t wgrid_smem_bytes(int win_rows, int win_cols, int chunk_values) {
  return wwindow_bytes(sizeof(real), win_rows, win_cols) +
         2 * band_stage_bytes<real>(chunk_values);
}

template <typename real>
cudaError_t launch_wdegrid(const WArgs<real> &a0, int ntasks, int win_rows, int win_cols,
                           cudaStream_t s) {
  if (ntasks == 0) return cudaSuccess;
  WArgs<real> a = a0;
  a.win_bytes = int(wwindow_bytes(sizeof(real), win_rows, win_cols));
  const size_t smem = wdegrid_smem_bytes<real>(win_rows, win_cols, a.chunk_values);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(
        wdegrid_band_kernel<real>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  wdegrid_band_kernel<real><<<ntasks, kBandWarps * 32, smem, s>>>(a);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_wgrid(const WArgs<real> &a0, int ntasks, int win_rows, int win_cols,
                         cudaStream_t s) {
  if (ntasks == 0) return cudaSuccess;
  WArgs<real> a = a0;
  a.win_bytes = int(wwindow_bytes(sizeof(real), win_rows, win_cols));
  const size_t smem = wgrid_smem_bytes<real>(win_rows, win_cols, a.chunk_values);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(
        wgrid_band_kernel<real>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  wgrid_band_kernel<real><<<ntasks, kBandWarps * 32, smem, s>>>(a);
  return cudaGetLastError();
}

template size_t wdegrid_smem_bytes<float>(int, int, int);
template size_t wdegrid_smem_bytes<double>(int, int, int);
template size_t wgrid_smem_bytes<float>(int, int, int);
template size_t wgrid_smem_bytes<double>(int, int, int);
template cudaError_t launch_wdegrid<float>(const WArgs<float> &, int, int, int, cudaStream_t);
template cudaError_t launch_wdegrid<double>(const WArgs<double> &, int, int, int, cudaStream_t);
template cudaError_t launch_wgrid<float>(const WArgs<float> &, int, int, int, cudaStream_t);
template cudaError_t launch_wgrid<double>(const WArgs<double> &, int, int, int, cudaStream_t);

}  // namespace pg
