// Device code shared by the single-operator and grouped (multi-channel)
// launches of the gridding kernels: tap evaluation, the
// asynchronous prologue copies, the G / G^H kernels and the fold of task
// windows.  Included by device_kernels.cu (GROUP = false) and
// batch_kernels.cu (GROUP = true), so each instantiation set compiles in its
// own translation unit.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "cplx_ops.cuh"
#include "pdl.cuh"
#include "device_kernels.h"
#include "plan.h"

namespace pg {
namespace dev {

// Tap weights of one axis by Horner's rule.  With SUB = false every lane
// reads the same coefficient at the same time, so the coefficients come
// straight from the constant bank of the kernel parameters.  Every kernel of
// the family is even, so tap J-1-j at x is (-1)^(J-1) times tap j at -x: the
// pair shares one evaluation split into even and odd parts,
// P_j(x) = E(x^2) + x O(x^2), P_{J-1-j}(x) = (-1)^(J-1) (E(x^2) - x O(x^2)).
//
// With SUB the lanes of a warp read the coefficients of different
// sub-segments.  From the parameter space those reads are served one
// address at a time, so the kernels first copy the coefficients into shared
// memory (stage_coefficients) and pass them as csm, laid out
// [j][s][c] -> csm[(j nsub + s) NC + c]: the lanes' sub-segments sit NC words
// apart, on different banks.
template <typename real, int J, bool SUB, int NC>
__device__ __forceinline__ void tap_weights(const PolyAxis<real, NC> &P, int nsub, real t,
                                            real (&k)[J], const real *csm = nullptr) {
  if (SUB) {
    const real ts = t * real(nsub);
    const int s = min(int(ts), nsub - 1);
    const real x = real(2) * (ts - real(s)) - real(1);
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const real *c = csm + (j * nsub + s) * NC;
      real acc = c[NC - 1];
#pragma unroll
      for (int i = NC - 2; i >= 0; --i) acc = fma(acc, x, c[i]);
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

// Tap weights of one axis over the register block of an item that spans G
// base cells along that axis (G = 1 or 2; block J + G - 1 cells).  With
// G = 2 the stored fraction x = t + d carries the visibility's cell d in
// {0, 1} inside the group: its J taps start at block cell d and the other
// block cell is 0.
template <typename real, int J, int G, bool SUB, int NC>
__device__ __forceinline__ void block_taps(const PolyAxis<real, NC> &P, int nsub, real x,
                                           real (&k)[J + G - 1], const real *csm = nullptr) {
  if constexpr (G == 1) {
    tap_weights<real, J, SUB>(P, nsub, x, k, csm);
  } else {
    const bool d = x >= real(1);
    real kk[J];
    tap_weights<real, J, SUB>(P, nsub, d ? x - real(1) : x, kk, csm);
    k[0] = d ? real(0) : kk[0];
#pragma unroll
    for (int j = 1; j < J; ++j) k[j] = d ? kk[j - 1] : kk[j];
    k[J] = d ? kk[J - 1] : real(0);
  }
}

// Copies the tap coefficients of the J taps and nsub sub-segments of P into
// csm (layout of tap_weights); the caller's next __syncthreads publishes
// them.  The register-block operators use one polynomial for both axes (one
// kernel, Ju == Jv), so one copy serves u and v.
template <typename real, int J, int NC>
__device__ __forceinline__ void stage_coefficients(const PolyAxis<real, NC> &P, int nsub,
                                                   real *csm) {
  const int n = J * nsub * NC;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int c = i % NC, js = i / NC;
    csm[i] = P.c[js / nsub][js % nsub][c];
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
// The same copy with an L2 evict-first policy, for streams read once (the
// coverage state): their lines leave L2 before those of the kernel's output.
template <int BYTES>
__device__ __forceinline__ void cp_async_stream(void *smem, const void *gmem,
                                                unsigned long long pol) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;\n" ::"r"(s),
                 "l"(gmem), "l"(pol)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], %2, %3;\n" ::"r"(s),
                 "l"(gmem), "n"(BYTES), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ unsigned long long l2_stream_policy() {
  unsigned long long p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Shared-memory layout of a task: the grid window(s), then the batch
// headers {first slot, kmax}, then the per-warp staging buffers.  The lane
// codes stay in global memory (L2): a warp reads its next batch's 32 codes
// (128 bytes, one load per lane) while it works on the current batch, so
// they cost no shared memory, which bounds the resident CTAs of small CTA
// shapes.
constexpr size_t kHeaderBytes = kMaxTaskBatches * sizeof(int2);
struct TaskHeaders {
  int2 *hdr;
  const int32_t *code;  // the task's lane codes, batch * 32 + lane (global)
};
// Issues the asynchronous copies of a task's batch headers; the caller waits
// with cp_async_wait_all() + __syncthreads().
template <typename A>
__device__ __forceinline__ TaskHeaders load_headers(const A &a, const Task &tk,
                                                    unsigned char *base) {
  TaskHeaders h;
  h.hdr = reinterpret_cast<int2 *>(base);
  h.code = a.lane_code + size_t(tk.batch_begin) * kBatch;
  const int nbt = tk.batch_end - tk.batch_begin;
  for (int k = threadIdx.x; k < nbt; k += blockDim.x)
    cp_async<8>(h.hdr + k, a.batches + tk.batch_begin + k);
  return h;
}
// Row and column of the packed index idx of a window WW cells wide, for a
// loop that advances idx by `step`: one division at the start instead of one
// per element.
struct WinCursor {
  int lp, lq, dp, dq;
  __device__ __forceinline__ WinCursor(int idx, int WW, int step) {
    lp = idx / WW;
    lq = idx - lp * WW;
    dp = step / WW;
    dq = step - dp * WW;
  }
  __device__ __forceinline__ void next(int WW) {
    lq += dq;
    lp += dp;
    if (lq >= WW) {
      lq -= WW;
      ++lp;
    }
  }
};
// Lane code of this lane in batch lb of a task (0, an empty item, past the
// task's last batch).
__device__ __forceinline__ int lane_code_at(const TaskHeaders &th, int lb, int nbt, int lane) {
  return lb < nbt ? __ldg(th.code + size_t(lb) * kBatch + lane) : 0;
}

// Visibility reads of the grid kernel.  Slot order: a streaming load of
// slot i.  Caller order: the gather of visibility m = slot_user[i] (0 for
// null slots, m < 0), at L2 evict-last priority when the launch keeps the
// caller-ordered vector in L2 (ApplyArgs::keep_in).
__device__ __forceinline__ unsigned long long l2_keep_policy() {
  unsigned long long p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ float2 load_keep(const float2 *p, unsigned long long pol) {
  float2 v;
  asm volatile("ld.global.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
               : "=f"(v.x), "=f"(v.y)
               : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ double2 load_keep(const double2 *p, unsigned long long pol) {
  double2 v;
  asm volatile("ld.global.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
               : "=d"(v.x), "=d"(v.y)
               : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ void store_keep(float2 *p, float2 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y),
               "l"(pol)
               : "memory");
}
__device__ __forceinline__ void store_keep(double2 *p, double2 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(p), "d"(v.x), "d"(v.y),
               "l"(pol)
               : "memory");
}
template <typename real>
__device__ __forceinline__ cplx<real> gather_vis(const cplx<real> *vin, int m, bool keep,
                                                unsigned long long pol) {
  if (m < 0) return cplx<real>{0, 0};
  return keep ? load_keep(vin + m, pol) : vin[m];
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

// Per-warp staging of the degrid kernel's coverage stream.  A warp walks its
// (batch, k) steps in chunks of CH steps, across batch boundaries; while it
// computes one chunk, the
// next chunk's per-slot data (t, and the caller index when the launch
// writes caller order) is on its way into shared memory by cp.async, so a
// whole chunk of loads is in flight per warp instead of one step.  Each lane
// copies and later reads only its own column, so the per-thread
// cp.async.wait_group is the only wait.  Layout per warp, each [2][CH][32]:
// t, then the caller index (int).  The grid kernel does not stage: its
// per-warp windows already fill shared memory, and staging would cost it
// resident CTAs.
//
// Weights are not applied in these kernels: the phase sign rides in t_u and
// operators with weights multiply by them in element-wise passes around the
// kernels.  (Instantiations that staged and applied a weight stream here
// raised "illegal instruction" on the GPU for some supports; see the design
// notes.)
template <typename real, int J>
struct StageDepth {
  static constexpr int value = (J <= 4 ? 4 : 8) / (sizeof(real) == 8 ? 2 : 1);
};
inline constexpr int stage_depth(int precision_bytes, int J) {
  return (J <= 4 ? 4 : 8) / (precision_bytes == 8 ? 2 : 1);
}

__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <typename real, int J, int G, bool SUB, bool GROUP>
__global__ void __launch_bounds__(256) degrid_kernel(const ApplyArgs<real> a0,
                                                     const __grid_constant__ PolyTable<real> poly) {
  using C = cplx<real>;
  constexpr int CH = StageDepth<real, J>::value;
  // register block of an item (group code G: group_u x group_v base cells)
  constexpr int JBU = J + group_u(G) - 1, JBV = J + group_v(G) - 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pdl_launch_next();
  const int task_id = a0.order ? a0.order[blockIdx.x] : int(blockIdx.x);
  const Task tk = a0.tasks[task_id];
  const auto &a = ArgsOf<real, GROUP>::get(a0, tk.channel);
  // the window in shared memory: WH rows of WW cells at row stride WS,
  // cell (r, c) at win_offset(r, c, WS, G)
  const int WW = tk.W + JBU - 1, WH = tk.H + JBV - 1, WS = a.win_stride;
  C *win = reinterpret_cast<C *>(smem_raw);
  const TaskHeaders th = load_headers(a, tk, smem_raw + a0.win_bytes);
  const C *grid = static_cast<const C *>(a.grid);
  const size_t ld = size_t(a.ld ? a.ld : a.Nu);
  // tap coefficients of sub-segmented kernels, after the staging buffers
  real *csm = reinterpret_cast<real *>(smem_raw + a0.win_bytes + kHeaderBytes +
                                       size_t(blockDim.x >> 5) * a0.stage_bytes);
  if (SUB) stage_coefficients<real, J>(poly.u, poly.nsub_u, csm);
  // the grid is the previous kernel's output
  pdl_wait();
  // Stage the (wrapped) window of the grid this tile's footprints touch.
  WinCursor cur(threadIdx.x, WW, blockDim.x);
  for (int idx = threadIdx.x; idx < WW * WH; idx += blockDim.x, cur.next(WW)) {
    const int lp = cur.lp, lq = cur.lq;
    int p = tk.P + lp;
    if (p >= a.Nv) p -= a.Nv;
    int q = tk.Q + lq;
    if (q >= a.Nu) q -= a.Nu;
    cp_async<sizeof(C)>(win + win_offset(lp, lq, WS, G), grid + size_t(p) * ld + q);
  }
  cp_async_wait_all();
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int nbt = tk.batch_end - tk.batch_begin;
  const C *frac = static_cast<const C *>(a.frac);
  const int32_t *user = a.slot_user;
  C *out = static_cast<C *>(a.slot_out);
  // caller-ordered output kept in L2 (evict-last) for the adjoint's gather
  const bool keep = a.keep_in != 0;
  if (warp >= nbt) return;
  unsigned char *stg = smem_raw + a0.win_bytes + kHeaderBytes + size_t(warp) * a0.stage_bytes;
  C *st_t = reinterpret_cast<C *>(stg);
  int *st_m = reinterpret_cast<int *>(stg + 2 * CH * 32 * sizeof(C));
  const unsigned long long pol = l2_stream_policy();
  const unsigned long long kpol = l2_keep_policy();
  // A chunk is the next CH (batch, k) steps of this warp, across batch
  // boundaries, so that a warp whose batches are short (one or two steps)
  // still has CH steps of coverage loads in flight.  The producer cursor
  // (plb, pk) issues chunk c + 1 while the compute cursor works on chunk c;
  // both take min(CH, steps left) steps per chunk, so they stay in step.
  auto issue = [&](int &lb, int &k, int buf) {
    for (int j = 0; j < CH && lb < nbt; ++j) {
      const size_t i = size_t(th.hdr[lb].x) + size_t(k) * kBatch + lane;
      const int e = (buf * CH + j) * 32 + lane;
      cp_async_stream<sizeof(C)>(st_t + e, frac + i, pol);
      if (user) cp_async_stream<4>(st_m + e, user + i, pol);
      if (++k >= th.hdr[lb].y) {
        k = 0;
        lb += nw;
      }
    }
    cp_async_commit();
  };
  int plb = warp, pk = 0;  // producer cursor: the next step to issue
  issue(plb, pk, 0);
  int lb = warp, k = 0, buf = 0, cnt = 0;
  int code_n = lane_code_at(th, lb, nbt, lane);  // lane code of batch lb
  C F[JBV][JBU];
  while (lb < nbt) {
    if (plb < nbt)
      issue(plb, pk, buf ^ 1);
    else
      cp_async_commit();  // empty group: keeps "all but the newest group" meaning this chunk
    cp_async_wait_group<1>();
    for (int j = 0; j < CH && lb < nbt; ++j) {
      const int2 bt = th.hdr[lb];
      if (k == 0) {
        // new batch: this lane's item and its J x J grid block; the code of
        // the warp's next batch is loaded now, to be ready when it starts
        const int code = code_n;
        code_n = lane_code_at(th, lb + nw, nbt, lane);
        cnt = item_count(code);
        const C *blk = win + win_offset(item_lp(code), item_lq(code), WS, G);
#pragma unroll
        for (int jv = 0; jv < JBV; ++jv)
#pragma unroll
          for (int ju = 0; ju < JBU; ++ju) F[jv][ju] = blk[win_offset(jv, ju, WS, G)];
      }
      const int e = (buf * CH + j) * 32 + lane;
      const C t = st_t[e];
      real ku[JBU], kv[JBV];
      block_taps<real, J, group_u(G), SUB>(poly.u, poly.nsub_u, fabs(t.x), ku, csm);
      block_taps<real, J, group_v(G), SUB>(poly.v, poly.nsub_v, t.y, kv, csm);
      C sum{0, 0};
#pragma unroll
      for (int jv = 0; jv < JBV; ++jv) {
        C row{0, 0};
#pragma unroll
        for (int ju = 0; ju < JBU; ++ju) row = fma2(splat(ku[ju]), F[jv][ju], row);
        sum = fma2(splat(kv[jv]), row, sum);
      }
      // the phase sign (-1)^(k_u + k_v) rides in the sign of t_u
      const real sg = copysign(real(1), t.x);
      const C y{sg * sum.x, sg * sum.y};
      // Lanes past their item's end compute on null slots: 0 in slot order,
      // nothing in caller order.
      if (!user) {
        out[size_t(bt.x) + size_t(k) * kBatch + lane] = k < cnt ? y : C{0, 0};
      } else {
        const int m = st_m[e];
        if (m >= 0) {
          if (keep)
            store_keep(out + m, y, kpol);
          else
            out[m] = y;
        }
      }
      if (++k >= bt.y) {
        k = 0;
        lb += nw;
      }
    }
    buf ^= 1;
  }
  cp_async_wait_all();
}

// Coverage loads the grid kernel keeps in flight per warp (depth, in steps)
// and how many steps before its gather a caller index is loaded
// (index_lead).  Wide supports: 2 and 1; a step's arithmetic covers the
// latencies and registers are short (deeper measured slower at J = 6).
// Below J = 6 the steps are short and registers to spare: 4 and 3.
// CALLER: the instantiation launched to gather caller order (FP32, J < 6);
// the slot-ordered launches keep 2 and 1, which measured faster there.
template <typename real, int J, bool CALLER>
struct GridAhead {
  static constexpr bool narrow = sizeof(real) == 4 && J < 6 && CALLER;
  static constexpr int depth = narrow ? 4 : 2;
  static constexpr int index_lead = narrow ? 3 : 1;
};

template <typename real, int J, int G, bool SUB, bool GROUP, bool CALLER = false>
__global__ void __launch_bounds__(256) grid_kernel(const ApplyArgs<real> a0,
                                                   const __grid_constant__ PolyTable<real> poly) {
  using C = cplx<real>;
  // register block of an item (group code G: group_u x group_v base cells)
  constexpr int JBU = J + group_u(G) - 1, JBV = J + group_v(G) - 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pdl_launch_next();
  const int task_id = a0.order ? a0.order[blockIdx.x] : int(blockIdx.x);
  const Task tk = a0.tasks[task_id];
  const auto &a = ArgsOf<real, GROUP>::get(a0, tk.channel);
  // warp windows in shared memory: WH rows at row stride WS (WN cells each,
  // cell (r, c) at win_offset(r, c, WS, G)); the task window written out is
  // WH x WW, packed
  const int WW = tk.W + JBU - 1, WH = tk.H + JBV - 1, WS = a.win_stride,
            WN = win_cells(WH, WS, G);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  C *wins = reinterpret_cast<C *>(smem_raw);
  const TaskHeaders th = load_headers(a, tk, smem_raw + a0.win_bytes);
  {
    // zero the warp windows, 16 bytes per store (the windows start 16-byte
    // aligned; an odd FP32 cell count leaves one 8-byte cell at the end)
    const size_t bytes = size_t(nw) * WN * sizeof(C);
    uint4 *z = reinterpret_cast<uint4 *>(smem_raw);
    for (int idx = threadIdx.x; idx < int(bytes / 16); idx += blockDim.x)
      z[idx] = make_uint4(0u, 0u, 0u, 0u);
    if (bytes % 16 != 0 && threadIdx.x == 0) wins[nw * WN - 1] = C{0, 0};
  }
  // tap coefficients of sub-segmented kernels, after the batch headers
  real *csm = reinterpret_cast<real *>(smem_raw + a0.win_bytes + kHeaderBytes);
  if (SUB) stage_coefficients<real, J>(poly.u, poly.nsub_u, csm);
  cp_async_wait_all();
  __syncthreads();
  // the visibilities are the previous kernel's output
  pdl_wait();
  C *mine = wins + warp * WN;
  const int nbt = tk.batch_end - tk.batch_begin;
  const C *frac = static_cast<const C *>(a.frac);
  const C *vin = static_cast<const C *>(a.slot_in);
  if (warp < nbt) {
    // Two cursors over this warp's (batch, k) steps, slot = hdr[lb].x +
    // 32 k + lane: the compute cursor and, two steps ahead of it, the
    // prefetch cursor, so two steps of coverage loads are in flight.  In
    // caller order the prefetch gathers vin[slot_user[slot]]; the caller
    // index of the prefetch cursor's slot is loaded one step before its
    // gather (mq), so a gather never waits on its index load.
    int clb = warp, ck = 0;
    int plb = warp, pk = 0;
    // lane codes of the compute cursor's batch and of the warp's next batch
    int code_c = lane_code_at(th, clb, nbt, lane);
    int code_n = lane_code_at(th, clb + nw, nbt, lane);
    auto adv = [&](int &lb, int &k) {
      if (k + 1 < th.hdr[lb].y) {
        ++k;
      } else {
        k = 0;
        lb += nw;
      }
    };
    auto slot = [&](int lb, int k) { return size_t(th.hdr[lb].x) + size_t(k) * kBatch + lane; };
    const int32_t *user = a.slot_user;
    const bool keep = a.keep_in != 0;
    const unsigned long long kpol = l2_keep_policy();
    auto index_at = [&](int lb, int k) { return lb < nbt ? __ldcs(user + slot(lb, k)) : -1; };
    auto value_at = [&](int lb, int k, int m) {
      return user ? gather_vis<real>(vin, m, keep, kpol) : __ldcs(vin + slot(lb, k));
    };
    // D steps of loads in flight (tq[0], yq[0]: the compute cursor's).  In
    // caller order a gather's index was loaded IL steps before it: IL = 1
    // keeps one index (mq) beside the prefetch cursor; IL > 1 runs an index
    // cursor (qlb, qk) IL - 1 steps past it, with the indices between in mr.
    constexpr int D = GridAhead<real, J, CALLER>::depth;
    constexpr int IL = GridAhead<real, J, CALLER>::index_lead;
    int mq = -1;
    int qlb = plb, qk = pk;
    int mr[IL];
    auto next_index = [&]() {
      int m = -1;
      if (qlb < nbt) {
        m = index_at(qlb, qk);
        adv(qlb, qk);
      }
      return m;
    };
    if constexpr (IL == 1) {
      mq = user ? index_at(plb, pk) : -1;
    } else {
#pragma unroll
      for (int i = 0; i < IL; ++i) mr[i] = user ? next_index() : -1;
    }
    auto prefetch = [&](C &t, C &y) {
      t = stream_load(frac + slot(plb, pk));
      if constexpr (IL == 1) {
        y = value_at(plb, pk, mq);
        adv(plb, pk);
        if (user) mq = index_at(plb, pk);
      } else {
        y = value_at(plb, pk, mr[0]);
        adv(plb, pk);
        if (user) {
#pragma unroll
          for (int i = 0; i + 1 < IL; ++i) mr[i] = mr[i + 1];
          mr[IL - 1] = next_index();
        }
      }
    };
    C tq[D], yq[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      tq[d] = C{0, 0};
      yq[d] = C{0, 0};
      if (d == 0 || plb < nbt) prefetch(tq[d], yq[d]);
    }
    C acc[JBV][JBU];
#pragma unroll
    for (int jv = 0; jv < JBV; ++jv)
#pragma unroll
      for (int ju = 0; ju < JBU; ++ju) acc[jv][ju] = C{0, 0};
    while (clb < nbt) {
      const C t = tq[0], yv = yq[0];
#pragma unroll
      for (int d = 0; d + 1 < D; ++d) {
        tq[d] = tq[d + 1];
        yq[d] = yq[d + 1];
      }
      if (plb < nbt) prefetch(tq[D - 1], yq[D - 1]);
      // Null slots hold a zero visibility, so they add nothing.  The phase
      // sign (-1)^(k_u + k_v) rides in the sign of t_u.
      const real sg = copysign(real(1), t.x);
      const real zr = sg * yv.x, zi = sg * yv.y;
      real ku[JBU], kv[JBV];
      block_taps<real, J, group_u(G), SUB>(poly.u, poly.nsub_u, fabs(t.x), ku, csm);
      block_taps<real, J, group_v(G), SUB>(poly.v, poly.nsub_v, t.y, kv, csm);
      const C z{zr, zi};
#pragma unroll
      for (int jv = 0; jv < JBV; ++jv) {
        const C az = mul2(z, splat(kv[jv]));
#pragma unroll
        for (int ju = 0; ju < JBU; ++ju) acc[jv][ju] = fma2(az, splat(ku[ju]), acc[jv][ju]);
      }
      if (ck + 1 >= th.hdr[clb].y) {
        // Flush at the end of the batch.  The items of one batch have
        // distinct base cells, so at each (jv, ju) step the 32 lanes update
        // 32 distinct cells; steps are ordered by __syncwarp, which makes the
        // summation order a function of the plan.
        const int code = code_c;
        code_c = code_n;
        code_n = lane_code_at(th, clb + 2 * nw, nbt, lane);
        const int cnt = item_count(code);
        C *blk = mine + win_offset(item_lp(code), item_lq(code), WS, G);
#pragma unroll
        for (int jv = 0; jv < JBV; ++jv)
#pragma unroll
          for (int ju = 0; ju < JBU; ++ju) {
            if (cnt > 0) {
              C *cell = blk + win_offset(jv, ju, WS, G);
              *cell = add2(*cell, acc[jv][ju]);
            }
            acc[jv][ju] = C{0, 0};
            __syncwarp();
          }
      }
      adv(clb, ck);
    }
  }
  __syncthreads();
  const int local_task = GROUP ? task_id - a0.group_task_base[tk.channel] : task_id;
  C *out = static_cast<C *>(a.tilebuf) + size_t(local_task) * a.slot_stride;
  WinCursor cur(threadIdx.x, WW, blockDim.x);
  for (int idx = threadIdx.x; idx < WW * WH; idx += blockDim.x, cur.next(WW)) {
    const int e = win_offset(cur.lp, cur.lq, WS, G);
    C s = wins[e];
    for (int w = 1; w < nw; ++w) {
      const C o = wins[w * WN + e];
      s.x += o.x;
      s.y += o.y;
    }
    out[idx] = s;
  }
}

// G^H G of the normal operator Phi^H Phi in one pass over each task (unit
// weights, single-cell items).  The task's grid window is staged in shared
// memory as in degrid_kernel, and the warp windows are zeroed as in
// grid_kernel.  Each lane keeps its item's J x J grid block F and its J x J
// accumulator block in registers.  Per visibility it evaluates the taps once,
// contracts them with F (the visibility degrid_kernel computes, in its order),
// and adds that value times the taps into the accumulator (grid_kernel's
// order; the two phase signs cancel).  Null slots add nothing.  Flushes,
// window sums and the task window written out are grid_kernel's.  So the
// task windows are those grid_kernel makes from degrid_kernel's slot-ordered
// output, bit for bit, without the slot-ordered vector and with one tap
// evaluation per visibility instead of two.  Shared memory: the grid window
// (a.stage_bytes bytes), the warp windows, then the batch headers at
// a.win_bytes.
template <typename real, int J, bool SUB>
__global__ void __launch_bounds__(256) normal_kernel(const ApplyArgs<real> a,
                                                     const __grid_constant__ PolyTable<real> poly) {
  using C = cplx<real>;
  constexpr int G = 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pdl_launch_next();
  const int task_id = a.order ? a.order[blockIdx.x] : int(blockIdx.x);
  const Task tk = a.tasks[task_id];
  const int WW = tk.W + J - 1, WH = tk.H + J - 1, WS = a.win_stride, WN = win_cells(WH, WS, G);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  C *gwin = reinterpret_cast<C *>(smem_raw);
  C *wins = reinterpret_cast<C *>(smem_raw + a.stage_bytes);
  const TaskHeaders th = load_headers(a, tk, smem_raw + a.win_bytes);
  {
    // zero the warp windows, 16 bytes per store (stage_bytes is a multiple
    // of 16; an odd FP32 cell count leaves one 8-byte cell at the end)
    const size_t bytes = size_t(nw) * WN * sizeof(C);
    uint4 *z = reinterpret_cast<uint4 *>(smem_raw + a.stage_bytes);
    for (int idx = threadIdx.x; idx < int(bytes / 16); idx += blockDim.x)
      z[idx] = make_uint4(0u, 0u, 0u, 0u);
    if (bytes % 16 != 0 && threadIdx.x == 0) wins[nw * WN - 1] = C{0, 0};
  }
  // tap coefficients of sub-segmented kernels, after the batch headers
  real *csm = reinterpret_cast<real *>(smem_raw + a.win_bytes + kHeaderBytes);
  if (SUB) stage_coefficients<real, J>(poly.u, poly.nsub_u, csm);
  const C *grid = static_cast<const C *>(a.grid);
  const size_t ld = size_t(a.ld ? a.ld : a.Nu);
  pdl_wait();  // the grid is the previous kernel's output
  WinCursor cur(threadIdx.x, WW, blockDim.x);
  for (int idx = threadIdx.x; idx < WW * WH; idx += blockDim.x, cur.next(WW)) {
    int p = tk.P + cur.lp;
    if (p >= a.Nv) p -= a.Nv;
    int q = tk.Q + cur.lq;
    if (q >= a.Nu) q -= a.Nu;
    cp_async<sizeof(C)>(gwin + win_offset(cur.lp, cur.lq, WS, G), grid + size_t(p) * ld + q);
  }
  cp_async_wait_all();
  __syncthreads();
  C *mine = wins + warp * WN;
  const int nbt = tk.batch_end - tk.batch_begin;
  const C *frac = static_cast<const C *>(a.frac);
  if (warp < nbt) {
    // compute cursor (clb, ck) and, two steps ahead, the prefetch cursor of
    // the fractions, as in grid_kernel
    int clb = warp, ck = 0;
    int plb = warp, pk = 0;
    int code_c = lane_code_at(th, clb, nbt, lane);
    int code_n = lane_code_at(th, clb + nw, nbt, lane);
    auto adv = [&](int &lb, int &k) {
      if (k + 1 < th.hdr[lb].y) {
        ++k;
      } else {
        k = 0;
        lb += nw;
      }
    };
    auto slot = [&](int lb, int k) { return size_t(th.hdr[lb].x) + size_t(k) * kBatch + lane; };
    C t0 = stream_load(frac + slot(plb, pk));
    adv(plb, pk);
    C t1{0, 0};
    if (plb < nbt) {
      t1 = stream_load(frac + slot(plb, pk));
      adv(plb, pk);
    }
    C F[J][J], acc[J][J];
    int cnt = 0;
    auto load_block = [&](int code) {
      cnt = item_count(code);
      const C *blk = gwin + win_offset(item_lp(code), item_lq(code), WS, G);
#pragma unroll
      for (int jv = 0; jv < J; ++jv)
#pragma unroll
        for (int ju = 0; ju < J; ++ju) F[jv][ju] = blk[win_offset(jv, ju, WS, G)];
    };
    load_block(code_c);
#pragma unroll
    for (int jv = 0; jv < J; ++jv)
#pragma unroll
      for (int ju = 0; ju < J; ++ju) acc[jv][ju] = C{0, 0};
    while (clb < nbt) {
      const C t = t0;
      t0 = t1;
      if (plb < nbt) {
        t1 = stream_load(frac + slot(plb, pk));
        adv(plb, pk);
      }
      real ku[J], kv[J];
      block_taps<real, J, 1, SUB>(poly.u, poly.nsub_u, fabs(t.x), ku, csm);
      block_taps<real, J, 1, SUB>(poly.v, poly.nsub_v, t.y, kv, csm);
      C sum{0, 0};
#pragma unroll
      for (int jv = 0; jv < J; ++jv) {
        C row{0, 0};
#pragma unroll
        for (int ju = 0; ju < J; ++ju) row = fma2(splat(ku[ju]), F[jv][ju], row);
        sum = fma2(splat(kv[jv]), row, sum);
      }
      if (ck < cnt) {
#pragma unroll
        for (int jv = 0; jv < J; ++jv) {
          const C az = mul2(sum, splat(kv[jv]));
#pragma unroll
          for (int ju = 0; ju < J; ++ju) acc[jv][ju] = fma2(az, splat(ku[ju]), acc[jv][ju]);
        }
      }
      if (ck + 1 >= th.hdr[clb].y) {
        // flush at the end of the batch, as grid_kernel does
        const int code = code_c;
        code_c = code_n;
        code_n = lane_code_at(th, clb + 2 * nw, nbt, lane);
        const int fcnt = item_count(code);
        C *blk = mine + win_offset(item_lp(code), item_lq(code), WS, G);
#pragma unroll
        for (int jv = 0; jv < J; ++jv)
#pragma unroll
          for (int ju = 0; ju < J; ++ju) {
            if (fcnt > 0) {
              C *cell = blk + win_offset(jv, ju, WS, G);
              *cell = add2(*cell, acc[jv][ju]);
            }
            acc[jv][ju] = C{0, 0};
            __syncwarp();
          }
        adv(clb, ck);
        if (clb < nbt) load_block(code_c);
      } else {
        adv(clb, ck);
      }
    }
  }
  __syncthreads();
  C *out = static_cast<C *>(a.tilebuf) + size_t(task_id) * a.slot_stride;
  WinCursor oc(threadIdx.x, WW, blockDim.x);
  for (int idx = threadIdx.x; idx < WW * WH; idx += blockDim.x, oc.next(WW)) {
    const int e = win_offset(oc.lp, oc.lq, WS, G);
    C s = wins[e];
    for (int w = 1; w < nw; ++w) {
      const C o = wins[w * WN + e];
      s.x += o.x;
      s.y += o.y;
    }
    out[idx] = s;
  }
}

// G^H on the column-walk plan, one CTA per task (an occupied tile), kWalkWarps
// warps with a shared-memory window each.  Warp w takes the tile's base-cell
// columns [w W / nw, (w + 1) W / nw); its lane r is row r.  Each lane keeps a
// J x J block of the window in registers that slides along its row: the
// block's physical column p holds window column q with q mod J = p.  At
// column q the lane adds the visibilities of base cell (r, q) (their taps
// reach columns q ... q + J - 1), then window column q is complete for this
// lane and is flushed: J read-modify-writes of cells (r + jv, q), one per
// step, steps ordered by __syncwarp.  In one step the 32 lanes touch 32
// distinct rows of one column, which an odd row stride spreads over every
// bank pair; a cell that two lanes reach (r + jv = r' + jv') is reached in
// different steps.  After its last column the warp flushes the J - 1
// columns its blocks still hold.  So a lane flushes J cells per column
// instead of J x J per work item.
//
// The warp first lists its steps in shared memory, one (first slot, active
// lanes) pair per (column, k), from its columns' counts; the main loop then
// keeps kWalkAhead steps of slot loads in flight across column boundaries.
// The windows are summed in warp order into the task's window, as in
// grid_kernel.
constexpr int kWalkAhead = 3;
constexpr int kWalkMaxCols = 8;  // columns of one warp: 32 / kWalkWarps
template <typename real, int J, bool SUB>
__global__ void __launch_bounds__(128, (sizeof(real) == 4 && J <= 6) ? 4 : 2) walk_grid_kernel(const WalkArgs<real> a,
                                                        const __grid_constant__ PolyTable<real> poly) {
  using C = cplx<real>;
  static_assert(kWalkMaxCols * kWalkWarps >= 32, "a warp's columns");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int task_id = a.order ? a.order[blockIdx.x] : int(blockIdx.x);
  const Task tk = a.tasks[task_id];
  const int WW = tk.W + J - 1, WH = tk.H + J - 1, WS = a.win_stride, WN = a.win_rows * WS;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  C *wins = reinterpret_cast<C *>(smem_raw);
  int2 *steps = reinterpret_cast<int2 *>(smem_raw + size_t(nw) * WN * sizeof(C)) +
                size_t(warp) * a.max_steps;
  int *colstep = reinterpret_cast<int *>(smem_raw + size_t(nw) * WN * sizeof(C) +
                                         size_t(nw) * a.max_steps * sizeof(int2)) +
                 warp * (kWalkMaxCols + 1);
  for (int idx = threadIdx.x; idx < nw * WN; idx += blockDim.x) wins[idx] = C{0, 0};
  // tap coefficients of sub-segmented kernels, after the step lists
  real *csm = reinterpret_cast<real *>(
      smem_raw + walk_coefficient_offset(sizeof(real), a.win_rows, WS, a.max_steps));
  if (SUB) stage_coefficients<real, J>(poly.u, poly.nsub_u, csm);
  C *mine = wins + warp * WN;
  const int q0 = warp * tk.W / nw, q1 = (warp + 1) * tk.W / nw;
  const unsigned lt = (1u << lane) - 1u;
  {
    // the warp's step list: the counts of its columns in flight together
    const int32_t *cnt = a.counts + size_t(task_id) * 32 * 32;
    int c[kWalkMaxCols];
#pragma unroll
    for (int i = 0; i < kWalkMaxCols; ++i) c[i] = q0 + i < q1 ? __ldg(cnt + (q0 + i) * 32 + lane) : 0;
    int base = q0 < q1 ? __ldg(a.colstart + size_t(task_id) * 33 + q0) : 0;
    int n = 0;
#pragma unroll
    for (int i = 0; i < kWalkMaxCols; ++i) {
      if (lane == 0) colstep[i] = n;
      const int kmax = __reduce_max_sync(0xffffffffu, c[i]);
      for (int k = 0; k < kmax; ++k) {
        const unsigned m = __ballot_sync(0xffffffffu, c[i] > k);
        if (lane == 0) steps[n] = make_int2(base, int(m));
        base += __popc(m);
        ++n;
      }
    }
    if (lane == 0) colstep[kWalkMaxCols] = n;
  }
  __syncthreads();
  const C *frac = static_cast<const C *>(a.frac);
  const C *vin = static_cast<const C *>(a.slot_in);
  const bool row_live = lane < tk.H;
  const int nsteps = colstep[kWalkMaxCols];
  // ring of the next kWalkAhead steps' loads
  C rt[kWalkAhead], ry[kWalkAhead];
  unsigned rm[kWalkAhead];
  auto fetch = [&](int j, C &t, C &y, unsigned &m) {
    m = 0;
    if (j < nsteps) {
      const int2 st = steps[j];
      m = unsigned(st.y);
      if ((m >> lane) & 1u) {
        const int slot = st.x + __popc(m & lt);
        t = stream_load(frac + slot);
        y = __ldcs(vin + slot);
      }
    }
  };
#pragma unroll
  for (int d = 0; d < kWalkAhead; ++d) {
    rt[d] = C{0, 0};
    ry[d] = C{0, 0};
    fetch(d, rt[d], ry[d], rm[d]);
  }
  int i = 0;
  C acc[J][J];
#pragma unroll
  for (int jv = 0; jv < J; ++jv)
#pragma unroll
    for (int p = 0; p < J; ++p) acc[jv][p] = C{0, 0};
  if (q0 < q1) {
    // columns qb, qb + 1, ... in blocks of J, so that a column's physical
    // block column (q mod J) is known at compile time in the unrolled body
    const int qb = q0 - q0 % J;
    for (int qq = qb; qq < q1 + J - 1; qq += J) {
#pragma unroll
      for (int p = 0; p < J; ++p) {
        const int q = qq + p;
        if (q >= q0 && q < q1) {
          const int end = colstep[q - q0 + 1];
          for (; i < end; ++i) {
            const C t = rt[0], yv = ry[0];
            const unsigned m = rm[0];
#pragma unroll
            for (int d = 0; d + 1 < kWalkAhead; ++d) {
              rt[d] = rt[d + 1];
              ry[d] = ry[d + 1];
              rm[d] = rm[d + 1];
            }
            fetch(i + kWalkAhead, rt[kWalkAhead - 1], ry[kWalkAhead - 1], rm[kWalkAhead - 1]);
            if ((m >> lane) & 1u) {
              const real sg = copysign(real(1), t.x);
              real ku[J], kv[J];
              tap_weights<real, J, SUB>(poly.u, poly.nsub_u, fabs(t.x), ku, csm);
              tap_weights<real, J, SUB>(poly.v, poly.nsub_v, t.y, kv, csm);
              const C z{sg * yv.x, sg * yv.y};
#pragma unroll
              for (int jv = 0; jv < J; ++jv) {
                const C az = mul2(z, splat(kv[jv]));
#pragma unroll
                for (int ju = 0; ju < J; ++ju)
                  acc[jv][(p + ju) % J] = fma2(az, splat(ku[ju]), acc[jv][(p + ju) % J]);
              }
            }
          }
        }
        if (q >= q0 && q < q1 + J - 1) {
          // window column q is complete: flush physical column p
#pragma unroll
          for (int jv = 0; jv < J; ++jv) {
            if (row_live) {
              C *cell = mine + (lane + jv) * WS + q;
              *cell = add2(*cell, acc[jv][p]);
            }
            acc[jv][p] = C{0, 0};
            __syncwarp();
          }
        }
      }
    }
  }
  __syncthreads();
  C *out = static_cast<C *>(a.tilebuf) + size_t(task_id) * a.slot_stride;
  WinCursor cur(threadIdx.x, WW, blockDim.x);
  for (int idx = threadIdx.x; idx < WW * WH; idx += blockDim.x, cur.next(WW)) {
    const int e = cur.lp * WS + cur.lq;
    C s = wins[e];
    for (int w = 1; w < nw; ++w) {
      const C o = wins[w * WN + e];
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
  // Launched with 32 x 8 threads: a thread owns column lq of a 32-column
  // chunk and rows ty, ty + 8, ty + 16, ty + 24 of a 32-row chunk, kept in
  // registers while the task windows are walked (outer loop over tasks).
  const int a = t / f.ntu, b = t - a * f.ntu;
  const int a2 = a == 0 ? f.ntv - 1 : a - 1;
  const int b2 = b == 0 ? f.ntu - 1 : b - 1;
  const int tu = a2 * f.ntu + b, tl = a * f.ntu + b2, td = a2 * f.ntu + b2;
  // independent broadcast loads of the tile's metadata
  const int P = f.tv_start[a], P1 = f.tv_start[a + 1], Q = f.tu_start[b], Q1 = f.tu_start[b + 1];
  const int Pu = f.tv_start[a2], Pu1 = f.tv_start[a2 + 1];
  const int Ql = f.tu_start[b2], Ql1 = f.tu_start[b2 + 1];
  const int own0 = f.tile_tasks[t], own1 = f.tile_tasks[t + 1];
  const int up0 = f.tile_tasks[tu], up1 = f.tile_tasks[tu + 1];
  const int lf0 = f.tile_tasks[tl], lf1 = f.tile_tasks[tl + 1];
  const int dg0 = f.tile_tasks[td], dg1 = f.tile_tasks[td + 1];
  const int H = P1 - P, W = Q1 - Q, Hu = Pu1 - Pu, Wl = Ql1 - Ql;
  const int WWo = W + f.Ju - 1, WWl = Wl + f.Ju - 1;
  const int64_t ss = f.slot_stride;
  const C *__restrict__ buf = static_cast<const C *>(f.tilebuf);
  C *__restrict__ grid = static_cast<C *>(f.grid);
  constexpr int R = 4;
  if (H == 32 && W == 32 && f.Jv <= 9 && f.Ju <= 33) {
    // Full tile, halos of at most 8 rows: thread (lq, ty) owns rows ty + 8 r
    // of column lq; a halo row ty < Jv - 1 is in r = 0 only.  The same sums
    // in the same order as below, with the per-row tests folded away and two
    // task windows' loads in flight.
    const int lq = int(threadIdx.x), ty = int(threadIdx.y);
    const bool top = ty < f.Jv - 1, left = lq < f.Ju - 1;
    C s[R];
#pragma unroll
    for (int r = 0; r < R; ++r) s[r] = C{0, 0};
    const C *own = buf + lq + ty * WWo;
#pragma unroll 2
    for (int k = own0; k < own1; ++k) {
      const C *w = own + k * ss;
      C v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = w[8 * r * WWo];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        s[r].x += v[r].x;
        s[r].y += v[r].y;
      }
    }
    if (top) {
      const C *up = buf + Hu * WWo + lq + ty * WWo;
      for (int k = up0; k < up1; ++k) {
        const C v = up[k * ss];
        s[0].x += v.x;
        s[0].y += v.y;
      }
    }
    if (left) {
      const C *lf = buf + lq + Wl + ty * WWl;
#pragma unroll 2
      for (int k = lf0; k < lf1; ++k) {
        const C *w = lf + k * ss;
        C v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = w[8 * r * WWl];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          s[r].x += v[r].x;
          s[r].y += v[r].y;
        }
      }
      if (top) {
        const C *dg = buf + Hu * WWl + lq + Wl + ty * WWl;
        for (int k = dg0; k < dg1; ++k) {
          const C v = dg[k * ss];
          s[0].x += v.x;
          s[0].y += v.y;
        }
      }
    }
    const size_t ld = size_t(f.ld ? f.ld : f.Nu);
    C *g = grid + (size_t(P) + ty) * ld + Q + lq;
#pragma unroll
    for (int r = 0; r < R; ++r) g[size_t(8 * r) * ld] = s[r];
    return;
  }
  for (int c0 = 0; c0 < W; c0 += 32) {
    const int lq = c0 + int(threadIdx.x);
    const bool col = lq < W, left = lq < f.Ju - 1;
    for (int r0 = 0; r0 < H; r0 += 8 * R) {
      C s[R];
      int lp[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        s[r] = C{0, 0};
        lp[r] = r0 + int(threadIdx.y) + 8 * r;
      }
      // own tile's task windows, in task order
      for (int k = own0; k < own1; ++k) {
        const C *w = buf + k * ss + lq;
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (col && lp[r] < H) {
            const C v = w[lp[r] * WWo];
            s[r].x += v.x;
            s[r].y += v.y;
          }
      }
      // halo rows of the tile above, then halo columns of the tile to the
      // left, then the corner of the tile above-left, each in task order
      if (r0 < f.Jv - 1)
        for (int k = up0; k < up1; ++k) {
          const C *w = buf + k * ss + Hu * WWo + lq;
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (col && lp[r] < f.Jv - 1 && lp[r] < H) {
              const C v = w[lp[r] * WWo];
              s[r].x += v.x;
              s[r].y += v.y;
            }
        }
      if (left)
        for (int k = lf0; k < lf1; ++k) {
          const C *w = buf + k * ss + lq + Wl;
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (lp[r] < H) {
              const C v = w[lp[r] * WWl];
              s[r].x += v.x;
              s[r].y += v.y;
            }
        }
      if (left && r0 < f.Jv - 1)
        for (int k = dg0; k < dg1; ++k) {
          const C *w = buf + k * ss + Hu * WWl + lq + Wl;
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (lp[r] < f.Jv - 1 && lp[r] < H) {
              const C v = w[lp[r] * WWl];
              s[r].x += v.x;
              s[r].y += v.y;
            }
        }
      if (col) {
        const size_t ld = size_t(f.ld ? f.ld : f.Nu);
        C *g = grid + size_t(P) * ld + Q + lq;
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (lp[r] < H) g[size_t(lp[r]) * ld] = s[r];
      }
    }
  }
}

// Per-warp staging bytes of the degrid kernel (see StageDepth): t, and the
// caller index if visibilities are written in caller order.
inline size_t stage_bytes(int precision_bytes, int J, bool user) {
  const size_t CH = size_t(stage_depth(precision_bytes, J));
  const size_t c = 2 * size_t(precision_bytes);
  return 2 * CH * 32 * (c + (user ? 4 : 0));
}

// Shared bytes of the tap coefficients a kernel with sub-segmented taps
// copies (stage_coefficients): J taps x nsub sub-segments x the precision's
// coefficient count; none without sub-segments.
inline size_t coefficient_bytes(int precision_bytes, int J, int nsub) {
  if (nsub <= 1) return 0;
  const size_t nc = precision_bytes == 8 ? PolyCount<double>::value : PolyCount<float>::value;
  return (size_t(J) * nsub * nc * precision_bytes + 15) / 16 * 16;
}
template <typename real>
inline int poly_nsub(const PolyTable<real> &poly) {
  return poly.nsub_u > poly.nsub_v ? poly.nsub_u : poly.nsub_v;
}

inline size_t window_bytes(int precision_bytes, int win_rows, int win_cols, const LaunchShape &shape,
                           bool per_warp, int group = 1) {
  const size_t one = size_t(win_cells(win_rows, win_cols, group)) * 2 * precision_bytes;
  const size_t b = per_warp ? one * size_t(shape.threads / 32) : one;
  return (b + 15) / 16 * 16;
}

// Dispatch on the support J (templated so the J x J block stays in registers)
// and on whether the kernel polynomial has sub-segments (narrow kernels, PSWF).

template <typename real, int J, int G, bool SUB, bool GROUP>
cudaError_t launch_one(bool degrid, const ApplyArgs<real> &a, const PolyTable<real> &poly,
                       int ntasks, size_t smem, int threads, cudaStream_t s) {
  auto fn = degrid ? degrid_kernel<real, J, G, SUB, GROUP> : grid_kernel<real, J, G, SUB, GROUP>;
  if constexpr (sizeof(real) == 4 && J < 6 && G == 1 && !GROUP) {
    // G^H gathering caller order at narrow supports: deeper prefetch
    if (!degrid && a.slot_user) fn = grid_kernel<real, J, G, SUB, GROUP, true>;
  }
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  return launch_chain(fn, dim3(ntasks), dim3(threads), smem, s, a, poly);
}

template <typename real, bool GROUP>
cudaError_t launch_apply(bool degrid, const ApplyArgs<real> &a, const PolyTable<real> &poly,
                         int J, int ntasks, size_t smem, int threads, cudaStream_t s) {
  if (ntasks == 0) return cudaSuccess;
  const bool sub = poly.nsub_u > 1 || poly.nsub_v > 1;
#define PG_CASE(JJ, GG)                                                                  \
  case JJ:                                                                               \
    return sub ? launch_one<real, JJ, GG, true, GROUP>(degrid, a, poly, ntasks, smem, threads, s) \
               : launch_one<real, JJ, GG, false, GROUP>(degrid, a, poly, ntasks, smem, threads, s);
  if (a.group_cells == 2) {
    // 2 x 2 groups: complex<float> with J <= kMaxGroupJ (the (J + 1)^2
    // block stays in registers)
    if constexpr (sizeof(real) == 4) {
      switch (J) {
        PG_CASE(1, 2)
        PG_CASE(2, 2)
        PG_CASE(3, 2)
        PG_CASE(4, 2)
        PG_CASE(5, 2)
        PG_CASE(6, 2)
      }
    }
    return cudaErrorInvalidValue;
  }
  if (a.group_cells == 3) {
    // pairs of cells of a row: complex<float> with J <= kMaxGroupJ (a
    // J x (J + 1) block)
    if constexpr (sizeof(real) == 4) {
      switch (J) {
        PG_CASE(1, 3)
        PG_CASE(2, 3)
        PG_CASE(3, 3)
        PG_CASE(4, 3)
        PG_CASE(5, 3)
        PG_CASE(6, 3)
      }
    }
    return cudaErrorInvalidValue;
  }
  switch (J) {
    PG_CASE(1, 1)
    PG_CASE(2, 1)
    PG_CASE(3, 1)
    PG_CASE(4, 1)
    PG_CASE(5, 1)
    PG_CASE(6, 1)
    PG_CASE(7, 1)
    PG_CASE(8, 1)
  }
#undef PG_CASE
  return cudaErrorInvalidValue;
}

}  // namespace dev
}  // namespace pg
