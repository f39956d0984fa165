// Device code shared by the single-operator and grouped (multi-channel)
// launches of the gridding kernels: complex types, tap evaluation, the
// asynchronous prologue copies, the G / G^H kernels and the fold of task
// windows.  Included by device_kernels.cu (GROUP = false) and
// batch_kernels.cu (GROUP = true), so each instantiation set compiles in its
// own translation unit.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "device_kernels.h"

namespace pg {
namespace dev {

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

// Tap weights of one axis by Horner's rule.  With SUB = false every lane
// reads the same coefficient at the same time, so the coefficients come
// straight from the constant bank of the kernel parameters.  Every kernel of
// the family is even, so tap J-1-j at x is (-1)^(J-1) times tap j at -x: the
// pair shares one evaluation split into even and odd parts,
// P_j(x) = E(x^2) + x O(x^2), P_{J-1-j}(x) = (-1)^(J-1) (E(x^2) - x O(x^2)).
template <typename real, int J, bool SUB, int NC>
__device__ __forceinline__ void tap_weights(const PolyAxis<real, NC> &P, int nsub, real t,
                                            real (&k)[J]) {
  if (SUB) {
    const real ts = t * real(nsub);
    const int s = min(int(ts), nsub - 1);
    const real x = real(2) * (ts - real(s)) - real(1);
#pragma unroll
    for (int j = 0; j < J; ++j) {
      real acc = P.c[j][s][NC - 1];
#pragma unroll
      for (int c = NC - 2; c >= 0; --c) acc = fma(acc, x, P.c[j][s][c]);
      k[j] = acc;
    }
    return;
  }
  const real x = real(2) * t - real(1);
  const real x2 = x * x;
  constexpr int NE = (NC + 1) / 2, NO = NC / 2;  // even / odd coefficient counts
#pragma unroll
  for (int j = 0; j < (J + 1) / 2; ++j) {
    real e = P.c[j][0][2 * (NE - 1)];
#pragma unroll
    for (int c = NE - 2; c >= 0; --c) e = fma(e, x2, P.c[j][0][2 * c]);
    real o = P.c[j][0][2 * NO - 1];
#pragma unroll
    for (int c = NO - 2; c >= 0; --c) o = fma(o, x2, P.c[j][0][2 * c + 1]);
    k[j] = fma(x, o, e);
    if (J - 1 - j != j) {
      const real mirror = fma(-x, o, e);
      k[J - 1 - j] = (J % 2 == 1) ? mirror : -mirror;
    }
  }
}

// Streaming loads of the coverage state: read once per apply, so they are
// marked evict-first and leave L2 to the visibility and grid data.
template <typename T>
__device__ __forceinline__ T stream_load(const T *p) {
  return __ldcs(p);
}

// Asynchronous global -> shared copies (cp.async): a CTA issues its whole
// prologue at once and waits one time, instead of one load latency per
// strided loop iteration.
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

// Shared-memory layout of a task: the grid window(s), then the batch
// headers {first slot, kmax} and the 32 lane codes of each batch.
struct TaskHeaders {
  int2 *hdr;
  int *code;
};
// Issues the asynchronous copies of a task's batch headers and lane codes;
// the caller waits with cp_async_wait_all() + __syncthreads().
template <typename A>
__device__ __forceinline__ TaskHeaders load_headers(const A &a, const Task &tk,
                                                    unsigned char *base) {
  TaskHeaders h;
  h.hdr = reinterpret_cast<int2 *>(base);
  h.code = reinterpret_cast<int *>(base + sizeof(int2) * kMaxTaskBatches);
  const int nbt = tk.batch_end - tk.batch_begin;
  for (int k = threadIdx.x; k < nbt; k += blockDim.x)
    cp_async<8>(h.hdr + k, a.batches + tk.batch_begin + k);
  // lane codes: 32 ints (128 bytes) per batch, copied in 16-byte pieces
  const int *src = a.lane_code + size_t(tk.batch_begin) * kBatch;
  for (int k = threadIdx.x; k < nbt * (kBatch / 4); k += blockDim.x)
    cp_async<16>(h.code + 4 * k, src + 4 * k);
  return h;
}

// Visibility read for the grid kernel: slot order, or caller order through
// slot_user (0 for null slots).
template <typename real>
__device__ __forceinline__ cplx<real> read_vis(const ApplyArgs<real> &a, const cplx<real> *vin,
                                              size_t i) {
  if (a.slot_user) {
    const int m = __ldcs(a.slot_user + i);
    return m >= 0 ? vin[m] : cplx<real>{0, 0};
  }
  return vin[i];
}

// Operator arguments of a task.  A single-operator launch reads them from the
// kernel parameters; a grouped launch (several operators in one grid) from
// the device table at a0.group, indexed by the task's channel.
template <typename real, bool GROUP>
struct ArgsOf {
  static __device__ __forceinline__ const ApplyArgs<real> &get(const ApplyArgs<real> &a0, int) {
    return a0;
  }
};
template <typename real>
struct ArgsOf<real, true> {
  static __device__ __forceinline__ ApplyArgs<real> get(const ApplyArgs<real> &a0, int ch) {
    return static_cast<const ApplyArgs<real> *>(a0.group)[ch];
  }
};

template <typename real, int J, bool SUB, bool GROUP>
__global__ void __launch_bounds__(256) degrid_kernel(const ApplyArgs<real> a0,
                                                     const __grid_constant__ PolyTable<real> poly) {
  using C = cplx<real>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Task tk = a0.tasks[blockIdx.x];
  const auto &a = ArgsOf<real, GROUP>::get(a0, tk.channel);
  const int WW = tk.W + J - 1, WH = tk.H + J - 1;
  C *win = reinterpret_cast<C *>(smem_raw);
  const TaskHeaders th = load_headers(a, tk, smem_raw + a0.win_bytes);
  const C *grid = static_cast<const C *>(a.grid);
  // Stage the (wrapped) window of the grid this tile's footprints touch.
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
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int nbt = tk.batch_end - tk.batch_begin;
  const C *frac = static_cast<const C *>(a.frac);
  const C *weight = static_cast<const C *>(a.weight);
  C *out = static_cast<C *>(a.slot_out);
  const bool unit = weight == nullptr;
  int lb = warp;
  if (lb >= nbt) return;
  // One flattened loop over (batch, k) per warp; the next slot's coverage
  // state is loaded one step ahead, across batch boundaries too.  Lanes past
  // their item's end compute on null slots, whose results are never read.
  int2 bt = th.hdr[lb];
  int k = 0;
  size_t i = size_t(bt.x) + lane;
  int cnt = item_count(th.code[lb * kBatch + lane]);
  C F[J][J];
  auto load_F = [&](int code) {
    const int lp = item_lp(code), lq = item_lq(code);
#pragma unroll
    for (int jv = 0; jv < J; ++jv)
#pragma unroll
      for (int ju = 0; ju < J; ++ju) F[jv][ju] = win[(lp + jv) * WW + lq + ju];
  };
  load_F(th.code[lb * kBatch + lane]);
  C t_next = stream_load(frac + i);
  int m_next = a.slot_user ? __ldcs(a.slot_user + i) : 0;
  while (true) {
    const C t = t_next;
    const int m = m_next;
    const size_t i_cur = i;
    const bool real_slot = k < cnt;  // null slots (past the lane's item) get 0
    // advance to the next slot of this warp
    bool new_batch = false;
    if (k + 1 < bt.y) {
      ++k;
      i += kBatch;
    } else {
      lb += nw;
      new_batch = true;
      if (lb < nbt) {
        bt = th.hdr[lb];
        k = 0;
        i = size_t(bt.x) + lane;
      }
    }
    const bool more = !new_batch || lb < nbt;
    if (more) {
      t_next = stream_load(frac + i);
      if (a.slot_user) m_next = __ldcs(a.slot_user + i);
    }
    real ku[J], kv[J];
    tap_weights<real, J, SUB>(poly.u, poly.nsub_u, fabs(t.x), ku);
    tap_weights<real, J, SUB>(poly.v, poly.nsub_v, t.y, kv);
    real sr = 0, si = 0;
#pragma unroll
    for (int jv = 0; jv < J; ++jv) {
      real rr = 0, ri = 0;
#pragma unroll
      for (int ju = 0; ju < J; ++ju) {
        rr = fma(ku[ju], F[jv][ju].x, rr);
        ri = fma(ku[ju], F[jv][ju].y, ri);
      }
      sr = fma(kv[jv], rr, sr);
      si = fma(kv[jv], ri, si);
    }
    C y;
    if (unit) {
      const real sg = copysign(real(1), t.x);
      y.x = sg * sr;
      y.y = sg * si;
    } else {
      const C w = stream_load(weight + i_cur);
      y.x = sr * w.x - si * w.y;
      y.y = sr * w.y + si * w.x;
    }
    if (!a.slot_user)
      out[i_cur] = real_slot ? y : C{0, 0};
    else if (m >= 0)
      out[m] = y;
    if (!more) break;
    if (new_batch) {
      const int code = th.code[lb * kBatch + lane];
      cnt = item_count(code);
      load_F(code);
    }
  }
}

template <typename real, int J, bool SUB, bool GROUP>
__global__ void __launch_bounds__(256) grid_kernel(const ApplyArgs<real> a0,
                                                   const __grid_constant__ PolyTable<real> poly) {
  using C = cplx<real>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Task tk = a0.tasks[blockIdx.x];
  const auto &a = ArgsOf<real, GROUP>::get(a0, tk.channel);
  const int WW = tk.W + J - 1, WH = tk.H + J - 1, WN = WW * WH;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  C *wins = reinterpret_cast<C *>(smem_raw);
  const TaskHeaders th = load_headers(a, tk, smem_raw + a0.win_bytes);
  for (int idx = threadIdx.x; idx < nw * WN; idx += blockDim.x) wins[idx] = C{0, 0};
  cp_async_wait_all();
  __syncthreads();
  C *mine = wins + warp * WN;
  const int nbt = tk.batch_end - tk.batch_begin;
  const C *frac = static_cast<const C *>(a.frac);
  const C *weight = static_cast<const C *>(a.weight);
  const C *vin = static_cast<const C *>(a.slot_in);
  const bool unit = weight == nullptr;
  int lb = warp;
  if (lb < nbt) {
    int2 bt = th.hdr[lb];
    int code = th.code[lb * kBatch + lane];
    int k = 0;
    size_t i = size_t(bt.x) + lane;
    C acc[J][J];
#pragma unroll
    for (int jv = 0; jv < J; ++jv)
#pragma unroll
      for (int ju = 0; ju < J; ++ju) acc[jv][ju] = C{0, 0};
    C t_next = stream_load(frac + i);
    C y_next = read_vis(a, vin, i);
    while (true) {
      const C t = t_next;
      const C yv = y_next;
      const size_t i_cur = i;
      bool new_batch = false;
      if (k + 1 < bt.y) {
        ++k;
        i += kBatch;
      } else {
        new_batch = true;
      }
      int2 bt_next = bt;
      if (new_batch && lb + nw < nbt) {
        bt_next = th.hdr[lb + nw];
        i = size_t(bt_next.x) + lane;
      }
      const bool more = !new_batch || lb + nw < nbt;
      if (more) {
        t_next = stream_load(frac + i);
        y_next = read_vis(a, vin, i);
      }
      // Null slots hold a zero visibility, so they add nothing.
      real zr, zi;
      if (unit) {
        const real sg = copysign(real(1), t.x);
        zr = sg * yv.x;
        zi = sg * yv.y;
      } else {
        // conj(weight) * y: G^H holds the conjugated entries of G.
        const C w = stream_load(weight + i_cur);
        zr = w.x * yv.x + w.y * yv.y;
        zi = w.x * yv.y - w.y * yv.x;
      }
      real ku[J], kv[J];
      tap_weights<real, J, SUB>(poly.u, poly.nsub_u, fabs(t.x), ku);
      tap_weights<real, J, SUB>(poly.v, poly.nsub_v, t.y, kv);
#pragma unroll
      for (int jv = 0; jv < J; ++jv) {
        const real ar = zr * kv[jv], ai = zi * kv[jv];
#pragma unroll
        for (int ju = 0; ju < J; ++ju) {
          acc[jv][ju].x = fma(ar, ku[ju], acc[jv][ju].x);
          acc[jv][ju].y = fma(ai, ku[ju], acc[jv][ju].y);
        }
      }
      if (new_batch) {
        // Flush.  The items of one batch have distinct base cells, so at each
        // (jv, ju) step the 32 lanes update 32 distinct cells; steps are
        // ordered by __syncwarp, which makes the summation order a function
        // of the plan.
        const int cnt = item_count(code);
        const int lp = item_lp(code), lq = item_lq(code);
#pragma unroll
        for (int jv = 0; jv < J; ++jv)
#pragma unroll
          for (int ju = 0; ju < J; ++ju) {
            if (cnt > 0) {
              C *cell = mine + (lp + jv) * WW + lq + ju;
              C c = *cell;
              c.x += acc[jv][ju].x;
              c.y += acc[jv][ju].y;
              *cell = c;
            }
            acc[jv][ju] = C{0, 0};
            __syncwarp();
          }
        lb += nw;
        if (!more) break;
        bt = bt_next;
        code = th.code[lb * kBatch + lane];
        k = 0;
      }
    }
  }
  __syncthreads();
  const int local_task = GROUP ? int(blockIdx.x) - a0.group_task_base[tk.channel] : int(blockIdx.x);
  C *out = static_cast<C *>(a.tilebuf) + size_t(local_task) * a.slot_stride;
  for (int idx = threadIdx.x; idx < WN; idx += blockDim.x) {
    C s = wins[idx];
    for (int w = 1; w < nw; ++w) {
      const C o = wins[w * WN + idx];
      s.x += o.x;
      s.y += o.y;
    }
    out[idx] = s;
  }
}

// One CTA per tile.  A cell sums, in this order, the windows of its own
// tile's tasks, then those of the tile above, the tile to the left and the
// tile above-left, where their J - 1 halo rows / columns reach into it.
template <typename real>
__device__ __forceinline__ void fold_tile(const FoldArgs &f, int t) {
  using C = cplx<real>;
  const int a = t / f.ntu, b = t - (t / f.ntu) * f.ntu;
  const int a2 = a == 0 ? f.ntv - 1 : a - 1;
  const int b2 = b == 0 ? f.ntu - 1 : b - 1;
  const int P = f.tv_start[a], Q = f.tu_start[b];
  const int H = f.tv_start[a + 1] - P, W = f.tu_start[b + 1] - Q;
  const int Hu = f.tv_start[a2 + 1] - f.tv_start[a2];  // height of the tile above
  const int Wl = f.tu_start[b2 + 1] - f.tu_start[b2];  // width of the tile to the left
  const int WWo = W + f.Ju - 1, WWl = Wl + f.Ju - 1;
  const int tu = a2 * f.ntu + b, tl = a * f.ntu + b2, td = a2 * f.ntu + b2;
  const int own0 = f.tile_tasks[t], own1 = f.tile_tasks[t + 1];
  const int up0 = f.tile_tasks[tu], up1 = f.tile_tasks[tu + 1];
  const int lf0 = f.tile_tasks[tl], lf1 = f.tile_tasks[tl + 1];
  const int dg0 = f.tile_tasks[td], dg1 = f.tile_tasks[td + 1];
  const C *__restrict__ buf = static_cast<const C *>(f.tilebuf);
  C *__restrict__ grid = static_cast<C *>(f.grid);
  auto cell_sum = [&](int idx) {
    const int lp = idx / W, lq = idx - lp * W;
    C s{0, 0};
    for (int k = own0; k < own1; ++k) {
      const C v = buf[size_t(k) * f.slot_stride + lp * WWo + lq];
      s.x += v.x;
      s.y += v.y;
    }
    const bool up = lp < f.Jv - 1, left = lq < f.Ju - 1;
    if (up)
      for (int k = up0; k < up1; ++k) {
        const C v = buf[size_t(k) * f.slot_stride + (lp + Hu) * WWo + lq];
        s.x += v.x;
        s.y += v.y;
      }
    if (left)
      for (int k = lf0; k < lf1; ++k) {
        const C v = buf[size_t(k) * f.slot_stride + lp * WWl + lq + Wl];
        s.x += v.x;
        s.y += v.y;
      }
    if (up && left)
      for (int k = dg0; k < dg1; ++k) {
        const C v = buf[size_t(k) * f.slot_stride + (lp + Hu) * WWl + lq + Wl];
        s.x += v.x;
        s.y += v.y;
      }
    return s;
  };
  // Four cells per thread per round, loads first, so their latencies overlap.
  constexpr int R = 4;
  for (int base = threadIdx.x; base < H * W; base += R * blockDim.x) {
    C s[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int idx = base + r * blockDim.x;
      if (idx < H * W) s[r] = cell_sum(idx);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int idx = base + r * blockDim.x;
      if (idx < H * W) {
        const int lp = idx / W, lq = idx - lp * W;
        grid[size_t(P + lp) * f.Nu + Q + lq] = s[r];
      }
    }
  }
}

inline size_t window_bytes(int precision_bytes, int win_rows, int win_cols, const LaunchShape &shape,
                    bool per_warp) {
  const size_t one = size_t(win_rows) * win_cols * 2 * precision_bytes;
  const size_t b = per_warp ? one * size_t(shape.threads / 32) : one;
  return (b + 15) / 16 * 16;
}
constexpr size_t kHeaderBytes = kMaxTaskBatches * (sizeof(int2) + kBatch * sizeof(int));

// Dispatch on the support J (templated so the J x J block stays in registers)
// and on whether the kernel polynomial has sub-segments (narrow kernels, PSWF).

template <typename real, int J, bool SUB, bool GROUP>
cudaError_t launch_one(bool degrid, const ApplyArgs<real> &a, const PolyTable<real> &poly,
                       int ntasks, size_t smem, int threads, cudaStream_t s) {
  auto fn = degrid ? degrid_kernel<real, J, SUB, GROUP> : grid_kernel<real, J, SUB, GROUP>;
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  fn<<<ntasks, threads, smem, s>>>(a, poly);
  return cudaGetLastError();
}

template <typename real, bool GROUP>
cudaError_t launch_apply(bool degrid, const ApplyArgs<real> &a, const PolyTable<real> &poly,
                         int J, int ntasks, size_t smem, int threads, cudaStream_t s) {
  if (ntasks == 0) return cudaSuccess;
  const bool sub = poly.nsub_u > 1 || poly.nsub_v > 1;
#define PG_CASE(JJ)                                                                    \
  case JJ:                                                                             \
    return sub ? launch_one<real, JJ, true, GROUP>(degrid, a, poly, ntasks, smem, threads, s) \
               : launch_one<real, JJ, false, GROUP>(degrid, a, poly, ntasks, smem, threads, s);
  switch (J) {
    PG_CASE(1)
    PG_CASE(2)
    PG_CASE(3)
    PG_CASE(4)
    PG_CASE(5)
    PG_CASE(6)
    PG_CASE(7)
    PG_CASE(8)
  }
#undef PG_CASE
  return cudaErrorInvalidValue;
}

}  // namespace dev
}  // namespace pg
