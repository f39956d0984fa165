// Fused row passes of the padded-grid FFT (see fft_kernels.h).
//
// Each pass is a Stockham auto-sort FFT of length N = 16^a * {1, 2, 4, 8} over
// V rows per CTA, 256 threads.  Stage s with radix R and sub-transform length
// Ns takes, for butterfly j < N / R, the inputs j + r N / R, multiplies input
// r by w^(r (j mod Ns)) with w = exp(-+2 pi i / (Ns R)), does an R-point DFT
// in registers and writes output r to (j / Ns) Ns R + (j mod Ns) + r Ns; after
// the last stage the row is in natural order.  The first stage reads global
// memory (with the padding and correction of the pass applied), the last
// writes it (keeping only the columns the pass needs); the stages in between
// go through shared memory, every thread reading all its inputs before a
// barrier and then writing its outputs.  Shared memory holds each row padded
// by one element every 32 against bank conflicts.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "device_kernels.h"
#include "fft_kernels.h"
#include "pdl.cuh"

namespace pg {
namespace {

constexpr int kFftThreads = 256;

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// times -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
// times exp(-+2 pi i / 8) and exp(-+6 pi i / 8)
template <bool INV>
__device__ __forceinline__ float2 mul_w8(float2 a) {
  constexpr float h = 0.70710678118654752f;
  return INV ? make_float2(h * (a.x - a.y), h * (a.x + a.y)) : make_float2(h * (a.x + a.y), h * (a.y - a.x));
}
template <bool INV>
__device__ __forceinline__ float2 mul_w8_3(float2 a) {
  constexpr float h = 0.70710678118654752f;
  return INV ? make_float2(-h * (a.x + a.y), h * (a.x - a.y)) : make_float2(h * (a.y - a.x), -h * (a.x + a.y));
}

// exp(-+2 pi i m / 16) for the 16-point DFT's inner twiddles (m = n2 k1).
template <bool INV>
__device__ __forceinline__ float2 w16(int m) {
  constexpr float c1 = 0.92387953251128676f, s1 = 0.38268343236508977f,
                  h = 0.70710678118654752f;
  float c = 1.f, sn = 0.f;  // cos, sin of 2 pi m / 16
  switch (m) {
    case 1: c = c1; sn = s1; break;
    case 2: c = h; sn = h; break;
    case 3: c = s1; sn = c1; break;
    case 4: c = 0.f; sn = 1.f; break;
    case 6: c = -h; sn = h; break;
    case 9: c = -c1; sn = -s1; break;
  }
  return make_float2(c, INV ? sn : -sn);
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float2 *v);

// 16-point DFT as 4 x 4: DFT-4 over n1 of v[4 n1 + n2] for each n2, times
// w16^(n2 k1), then DFT-4 over n2 for each k1 into X[k1 + 4 k2].
template <bool INV>
__device__ __forceinline__ void dft16(float2 *v) {
  float2 a[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    float2 t[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
    dft<4, INV>(t);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) a[n2][k1] = (n2 && k1) ? cmulf(t[k1], w16<INV>(n2 * k1)) : t[k1];
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 t[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
    dft<4, INV>(t);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
  }
}

// Natural-order R-point DFT in registers, X_k = sum_m v_m exp(-+2 pi i m k / R).
template <int R, bool INV>
__device__ __forceinline__ void dft(float2 *v) {
  if constexpr (R == 16) {
    dft16<INV>(v);
  } else if constexpr (R == 2) {
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (R == 4) {
    const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    const float2 t2 = cadd(v[1], v[3]), t3 = mul_mi<INV>(csub(v[1], v[3]));
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  } else {
    static_assert(R == 8, "radix 2, 4, 8 or 16");
    float2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft<4, INV>(e);
    dft<4, INV>(o);
    o[1] = mul_w8<INV>(o[1]);
    o[2] = mul_mi<INV>(o[2]);
    o[3] = mul_w8_3<INV>(o[3]);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = cadd(e[k], o[k]);
      v[k + 4] = csub(e[k], o[k]);
    }
  }
}

// Row j of the image is row y0 + j of the padded grid.  Forward: image row
// (S applied) placed at columns x0 ... -> grid row.  Inverse: grid row ->
// image row (columns x0 ..., S applied).
template <bool INV>
__device__ __forceinline__ float2 load_in(const FftArgs &a, const float2 *__restrict__ in, int j,
                                          int n) {
  if (j >= a.Ny) return make_float2(0.f, 0.f);
  if constexpr (!INV) {
    const int i = n - a.x0;
    if (i < 0 || i >= a.Nx) return make_float2(0.f, 0.f);
    const float s = a.su[i] * a.sv[j];
    const float2 x = in[size_t(j) * a.Nx + i];
    return make_float2(s * x.x, s * x.y);
  } else {
    return in[size_t(a.y0 + j) * a.ld + n];
  }
}

template <bool INV>
__device__ __forceinline__ void store_out(const FftArgs &a, float2 *__restrict__ out, int j, int n,
                                          float2 v) {
  if (j >= a.Ny) return;
  if constexpr (!INV) {
    out[size_t(a.y0 + j) * a.ld + n] = v;
  } else {
    const int i = n - a.x0;
    if (i >= 0 && i < a.Nx) {
      const float s = a.su[i] * a.sv[j];
      out[size_t(j) * a.Nx + i] = make_float2(s * v.x, s * v.y);
    }
  }
}

// Shared-memory slot of element n of row `row`: one pad element every 32,
// and rows PAD elements further apart (the column pass picks PAD so that the
// V rows it reads at one n fall on different banks).
template <int N, int PAD = 0>
__device__ __forceinline__ int sidx(int row, int n) {
  constexpr int NP = N + N / 32 + PAD;
  return row * NP + n + (n >> 5);
}

// Twiddles w^r, r = 1 ... R-1, of w = exp(-+2 pi i k / (Ns R)) from w, w^2
// and w^4 (loaded from the table): the others as one product of two of them.
template <int R>
__device__ __forceinline__ void twiddle(float2 *v, const float2 (&w)[4]) {
  // w^r from the loaded powers w^(2^e): the product over the set bits of r
  float2 p[R];
  p[1] = w[0];
#pragma unroll
  for (int r = 2; r < R; ++r) {
    const int top = 31 - __clz(r), low = r - (1 << top);  // compile-time after unrolling
    p[r] = low ? cmulf(p[low], w[top]) : w[top];
  }
#pragma unroll
  for (int r = 1; r < R; ++r) v[r] = cmulf(v[r], p[r]);
}

// The twiddles of every stage after the first, loaded in the prologue
// together with the first stage's data so that one load latency covers them.
constexpr int kMaxStages = 4, kMaxQ = 8, kMaxPow = 4;
struct TwiddleCache {
  float2 w[kMaxStages][kMaxQ][kMaxPow];
};

// Radix of the stage with sub-transform length Ns: 16 while it divides the
// rest, then the remainder (2, 4 or 8).
template <int N, int Ns>
struct StageRadix {
  static constexpr int rem = N / Ns;
  static constexpr int value = rem % 16 == 0 ? 16 : rem;
};

template <int N, int V, int Ns, int S, bool INV, int T = kFftThreads, bool COLIO = false>
__device__ __forceinline__ void load_twiddles(TwiddleCache &c, const float2 *__restrict__ tw) {
  constexpr int R = StageRadix<N, Ns>::value;
  constexpr int NB = V * (N / R);
  constexpr int Q = (NB + T - 1) / T;
  static_assert(S < kMaxStages && Q <= kMaxQ, "twiddle cache size");
  if constexpr (Ns > 1) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int flat = int(threadIdx.x) + q * T;
      // the last stage of a column pass takes its butterflies column-fastest
      const int j = (COLIO && Ns * R == N) ? flat / V : flat % (N / R);
      const int step = (j % Ns) * (N / (Ns * R));
#pragma unroll
      for (int e = 0; e < kMaxPow; ++e) {
        if ((1 << e) < R && flat < NB) {
          float2 w = __ldg(tw + (step << e));
          if (INV) w.y = -w.y;
          c.w[S][q][e] = w;
        }
      }
    }
  }
  if constexpr (Ns * R < N) load_twiddles<N, V, Ns * R, S + 1, INV, T, COLIO>(c, tw);
}

// Stage S (sub-transform length Ns) of an N-point transform of V rows.  With
// COLIO the V "rows" are
// V adjacent columns of a grid with row stride a.ld starting at column row0:
// the first and last stages take their butterflies column-fastest (thread
// flat -> column flat mod V, butterfly flat / V), so that the V threads of a
// butterfly index read or write one contiguous V x 8-byte row segment; the
// first stage reads only rows a.y0 ... a.y0+a.Ny-1 (forward), the last writes
// only those rows (inverse).  Otherwise the first and last stages go through
// load_in / store_out.
template <int N, int V, int Ns, int S, bool INV, int PAD = 0, int T = kFftThreads,
          bool COLIO = false>
__device__ __forceinline__ void run_stages(const FftArgs &a, const float2 *__restrict__ in,
                                           float2 *__restrict__ out, float2 *sm,
                                           const TwiddleCache &tc, int row0) {
  constexpr int R = StageRadix<N, Ns>::value;
  constexpr bool FIRST = Ns == 1, LAST = Ns * R == N;
  constexpr int NB = V * (N / R);  // butterflies of the stage
  constexpr int Q = (NB + T - 1) / T;
  const int tid = threadIdx.x;
  float2 v[Q][R];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int flat = tid + q * T;
    if (flat < NB) {
      // column-fastest butterflies in the first and last stages of a column pass
      const bool cm = COLIO && (FIRST || LAST);
      const int rr = cm ? flat % V : flat / (N / R), j = cm ? flat / V : flat % (N / R);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int n = j + r * (N / R);
        if constexpr (FIRST && COLIO)
          v[q][r] = (INV || (n >= a.y0 && n < a.y0 + a.Ny))
                        ? in[size_t(n) * a.ld + row0 + rr]
                        : make_float2(0.f, 0.f);
        else if constexpr (FIRST)
          v[q][r] = load_in<INV>(a, in, row0 + rr, n);
        else
          v[q][r] = sm[sidx<N, PAD>(rr, n)];
      }
    }
  }
  if constexpr (!FIRST) __syncthreads();  // every read of this stage is done
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int flat = tid + q * T;
    if (flat < NB) {
      const bool cm = COLIO && (FIRST || LAST);
      const int rr = cm ? flat % V : flat / (N / R), j = cm ? flat / V : flat % (N / R);
      const int k = j % Ns;
      if constexpr (!FIRST) twiddle<R>(v[q], tc.w[S][q]);
      dft<R, INV>(v[q]);
      const int d = (j / Ns) * Ns * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int n = d + r * Ns;
        if constexpr (LAST && COLIO) {
          if (!INV || (n >= a.y0 && n < a.y0 + a.Ny)) out[size_t(n) * a.ld + row0 + rr] = v[q][r];
        } else if constexpr (LAST) {
          store_out<INV>(a, out, row0 + rr, n, v[q][r]);
        } else {
          sm[sidx<N, PAD>(rr, n)] = v[q][r];
        }
      }
    }
  }
  if constexpr (!LAST) {
    __syncthreads();
    run_stages<N, V, Ns * R, S + 1, INV, PAD, T, COLIO>(a, in, out, sm, tc, row0);
  }
}

template <int N, int V, bool INV>
__global__ void __launch_bounds__(kFftThreads, 4) fft_row_kernel(const FftArgs a,
                                                              const float2 *__restrict__ in,
                                                              float2 *__restrict__ out) {
  extern __shared__ float2 fft_sm[];
  dev::pdl_launch_next();
  TwiddleCache tc;
  load_twiddles<N, V, 1, 0, INV>(tc, static_cast<const float2 *>(a.tw_u));
  dev::pdl_wait();  // `in` is the previous kernel's output
  run_stages<N, V, 1, 0, INV>(a, in, out, fft_sm, tc, int(blockIdx.x) * V);
}

// One size group of a batch: member blockIdx.y's arguments from the channel
// table; the CTAs past that member's last row return at once.
template <int N, int V, bool INV>
__global__ void __launch_bounds__(kFftThreads, 4) fft_row_group_kernel(
    const ChannelIO<float> *__restrict__ chans, const int *__restrict__ members, int ld,
    const float2 *__restrict__ tw) {
  extern __shared__ float2 fft_sm[];
  const ChannelIO<float> &c = chans[members[blockIdx.y]];
  if (int(blockIdx.x) * V >= c.Ny) return;
  FftArgs a;
  a.Nx = c.Nx;
  a.Ny = c.Ny;
  a.Nu = c.Nu;
  a.Nv = c.Nv;
  a.x0 = c.x0;
  a.y0 = c.y0;
  a.ld = ld;
  a.su = c.su;
  a.sv = c.sv;
  const float2 *in = static_cast<const float2 *>(INV ? c.work : c.x_in);
  float2 *out = static_cast<float2 *>(INV ? c.x_out : c.pad);
  TwiddleCache tc;
  load_twiddles<N, V, 1, 0, INV>(tc, tw);
  run_stages<N, V, 1, 0, INV>(a, in, out, fft_sm, tc, int(blockIdx.x) * V);
}

// Column pass: V adjacent columns per CTA, so that every row of the block is
// one contiguous V x 8-byte segment.  The first stage reads the block's rows
// from global memory and the last stage writes them, both with the column
// index fastest across threads (run_stages COLIO); the stages in between run
// on the V columns as V rows of shared memory.  Forward: only rows y0 ...
// y0+Ny-1 of the input are read (the others are zero), all Nv rows are
// written.  Inverse: all rows are read, only rows y0 ... y0+Ny-1 are written.
// With a member table, the CTA's channel (column / Nu) gives y0 and Ny.
// V = 8 columns (64-byte row segments) from 256 rows up, 16 below; 512
// threads once the block holds 16K points, so that each thread keeps two
// radix-16 butterflies in registers.  Measured on 2048 x 2048 (forward /
// inverse): 8 columns and 512 threads 22.6 / 21.5 us per pass, 4 columns and
// 256 threads 24.6 / 24.2 us, 2 columns 30.9 / 28.4 us; cuFFT's strided
// plan 25.2 / 25.2 us; the same shapes with copy-in and copy-out passes
// through shared memory 25.5 / 24.3 us.
constexpr int col_block(int N) { return N >= 256 ? 8 : 16; }
constexpr int col_threads(int N) { return col_block(N) * N >= 16384 ? 512 : 256; }
template <int N, int V>
struct ColPad {
  // rows of the block sit 16 / V banks (8-byte units) apart
  static constexpr int value = ((16 / V) - (N + N / 32) % 16 + 16) % 16;
};

// The column pass with its first and last stages on global memory directly
// (run_stages COLIO): no copy-in and copy-out passes through shared memory.
template <int N, int V, bool INV, int T, int MINB>
__global__ void __launch_bounds__(T, MINB) fft_col_direct_kernel(const FftColArgs c) {
  extern __shared__ float2 fft_sm[];
  dev::pdl_launch_next();
  constexpr int PAD = ColPad<N, V>::value;
  const int col0 = int(blockIdx.x) * V;
  FftArgs a;
  a.y0 = c.y0;
  a.Ny = c.Ny;
  a.ld = c.ld;
  if (c.members) {
    const ChannelIO<float> &io =
        static_cast<const ChannelIO<float> *>(c.chans)[c.members[col0 / c.Nu]];
    a.y0 = io.y0;
    a.Ny = io.Ny;
  }
  TwiddleCache tc;
  load_twiddles<N, V, 1, 0, INV, T, true>(tc, static_cast<const float2 *>(c.tw_v));
  dev::pdl_wait();  // c.in is the previous kernel's output
  run_stages<N, V, 1, 0, INV, PAD, T, true>(a, static_cast<const float2 *>(c.in),
                                                   static_cast<float2 *>(c.out), fft_sm, tc,
                                                   col0);
}

template <int N, bool INV>
cudaError_t launch_cols(const FftColArgs &c, cudaStream_t s) {
  constexpr int V = col_block(N), T = col_threads(N);
  constexpr int PAD = ColPad<N, V>::value;
  const size_t smem = sizeof(float2) * size_t(V) * (N + N / 32 + PAD);
  auto fn = fft_col_direct_kernel<N, V, INV, T, T == 512 ? 1 : 2>;
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  return launch_chain(fn, dim3(c.W / V), dim3(T), smem, s, c);
}

template <bool INV>
cudaError_t launch_cols_n(const FftColArgs &c, cudaStream_t s) {
  switch (c.Nv) {
    case 64: return launch_cols<64, INV>(c, s);
    case 128: return launch_cols<128, INV>(c, s);
    case 256: return launch_cols<256, INV>(c, s);
    case 512: return launch_cols<512, INV>(c, s);
    case 1024: return launch_cols<1024, INV>(c, s);
    case 2048: return launch_cols<2048, INV>(c, s);
  }
  return cudaErrorInvalidValue;
}

// Rows per CTA: enough to give every thread a butterfly in the first
// (radix-16) stage.
constexpr int rows_per_cta(int N) { return N >= 4096 ? 1 : 4096 / N; }

template <int N, bool INV>
cudaError_t launch_rows(const FftArgs &a, const void *in, void *out, cudaStream_t s) {
  constexpr int V = rows_per_cta(N);
  const size_t smem = sizeof(float2) * size_t(V) * (N + N / 32);
  auto fn = fft_row_kernel<N, V, INV>;
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  return launch_chain(fn, dim3((a.Ny + V - 1) / V), dim3(kFftThreads), smem, s, a,
                      static_cast<const float2 *>(in), static_cast<float2 *>(out));
}

template <bool INV>
cudaError_t launch_n(const FftArgs &a0, const void *in, void *out, cudaStream_t s) {
  if (a0.Ny == 0) return cudaSuccess;
  FftArgs a = a0;
  if (a.ld == 0) a.ld = a.Nu;
  switch (a.Nu) {
    case 64: return launch_rows<64, INV>(a, in, out, s);
    case 128: return launch_rows<128, INV>(a, in, out, s);
    case 256: return launch_rows<256, INV>(a, in, out, s);
    case 512: return launch_rows<512, INV>(a, in, out, s);
    case 1024: return launch_rows<1024, INV>(a, in, out, s);
    case 2048: return launch_rows<2048, INV>(a, in, out, s);
    case 4096: return launch_rows<4096, INV>(a, in, out, s);
  }
  return cudaErrorInvalidValue;
}

template <int N, bool INV>
cudaError_t launch_group(const ChannelIO<float> *chans, const int *members, int nmembers,
                         int max_ny, int ld, const void *tw, cudaStream_t s) {
  constexpr int V = rows_per_cta(N);
  const size_t smem = sizeof(float2) * size_t(V) * (N + N / 32);
  auto fn = fft_row_group_kernel<N, V, INV>;
  if (smem > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  const dim3 grid((max_ny + V - 1) / V, nmembers);
  fn<<<grid, kFftThreads, smem, s>>>(chans, members, ld, static_cast<const float2 *>(tw));
  return cudaGetLastError();
}

template <bool INV>
cudaError_t launch_group_n(const ChannelIO<float> *chans, const int *members, int nmembers,
                           int Nu, int max_ny, int ld, const void *tw, cudaStream_t s) {
  switch (Nu) {
    case 64: return launch_group<64, INV>(chans, members, nmembers, max_ny, ld, tw, s);
    case 128: return launch_group<128, INV>(chans, members, nmembers, max_ny, ld, tw, s);
    case 256: return launch_group<256, INV>(chans, members, nmembers, max_ny, ld, tw, s);
    case 512: return launch_group<512, INV>(chans, members, nmembers, max_ny, ld, tw, s);
    case 1024: return launch_group<1024, INV>(chans, members, nmembers, max_ny, ld, tw, s);
    case 2048: return launch_group<2048, INV>(chans, members, nmembers, max_ny, ld, tw, s);
    case 4096: return launch_group<4096, INV>(chans, members, nmembers, max_ny, ld, tw, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

bool fft_rows_supported(int Nu) { return Nu >= 64 && Nu <= 4096 && (Nu & (Nu - 1)) == 0; }

std::vector<float> fft_twiddles(int N) {
  std::vector<float> t(2 * size_t(N));
  const double pi = 3.14159265358979323846;
  for (int m = 0; m < N; ++m) {
    const double ang = -2.0 * pi * double(m) / double(N);
    t[2 * size_t(m)] = float(std::cos(ang));
    t[2 * size_t(m) + 1] = float(std::sin(ang));
  }
  return t;
}

cudaError_t launch_fft_rows_forward(const FftArgs &a, const void *x, void *grid, cudaStream_t s) {
  if (!fft_rows_supported(a.Nu)) return cudaErrorInvalidValue;
  return launch_n<false>(a, x, grid, s);
}

cudaError_t launch_fft_rows_inverse(const FftArgs &a, const void *grid, void *x, cudaStream_t s) {
  if (!fft_rows_supported(a.Nu)) return cudaErrorInvalidValue;
  return launch_n<true>(a, grid, x, s);
}

bool fft_cols_supported(int Nv, int W) {
  // at 4096 rows the block's registers would spill
  if (!fft_rows_supported(Nv) || Nv > 2048 || W <= 0) return false;
  return W % (Nv >= 256 ? 8 : 16) == 0;
}

cudaError_t launch_fft_cols(bool inverse, const FftColArgs &c, cudaStream_t s) {
  if (!fft_cols_supported(c.Nv, c.W) || c.ld < c.W || (c.members && c.Nu <= 0) ||
      (!c.members && (c.y0 < 0 || c.Ny < 0 || c.y0 + c.Ny > c.Nv)))
    return cudaErrorInvalidValue;
  return inverse ? launch_cols_n<true>(c, s) : launch_cols_n<false>(c, s);
}

cudaError_t launch_fft_rows_group(bool inverse, const void *chans, const int *members, int nmembers,
                                  int Nu, int max_ny, int ld, const void *tw_u, cudaStream_t s) {
  if (!fft_rows_supported(Nu) || ld < Nu || nmembers < 0 || nmembers > 65535)
    return cudaErrorInvalidValue;
  if (nmembers == 0 || max_ny == 0) return cudaSuccess;
  const auto *c = static_cast<const ChannelIO<float> *>(chans);
  return inverse ? launch_group_n<true>(c, members, nmembers, Nu, max_ny, ld, tw_u, s)
                 : launch_group_n<false>(c, members, nmembers, Nu, max_ny, ld, tw_u, s);
}

}  // namespace pg
