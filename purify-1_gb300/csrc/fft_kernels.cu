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

#include "fft_kernels.h"

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
    return in[size_t(a.y0 + j) * a.Nu + n];
  }
}

template <bool INV>
__device__ __forceinline__ void store_out(const FftArgs &a, float2 *__restrict__ out, int j, int n,
                                          float2 v) {
  if (j >= a.Ny) return;
  if constexpr (!INV) {
    out[size_t(a.y0 + j) * a.Nu + n] = v;
  } else {
    const int i = n - a.x0;
    if (i >= 0 && i < a.Nx) {
      const float s = a.su[i] * a.sv[j];
      out[size_t(j) * a.Nx + i] = make_float2(s * v.x, s * v.y);
    }
  }
}

template <int N>
__device__ __forceinline__ int sidx(int row, int n) {
  constexpr int NP = N + N / 32;
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

template <int N, int V, int Ns, int S, bool INV>
__device__ __forceinline__ void load_twiddles(TwiddleCache &c, const float2 *__restrict__ tw) {
  constexpr int R = StageRadix<N, Ns>::value;
  constexpr int NB = V * (N / R);
  constexpr int Q = (NB + kFftThreads - 1) / kFftThreads;
  static_assert(S < kMaxStages && Q <= kMaxQ, "twiddle cache size");
  if constexpr (Ns > 1) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int flat = int(threadIdx.x) + q * kFftThreads;
      const int j = flat % (N / R);
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
  if constexpr (Ns * R < N) load_twiddles<N, V, Ns * R, S + 1, INV>(c, tw);
}

// Stage S (sub-transform length Ns) of an N-point transform of V rows.
template <int N, int V, int Ns, int S, bool INV>
__device__ __forceinline__ void run_stages(const FftArgs &a, const float2 *__restrict__ in,
                                           float2 *__restrict__ out, float2 *sm,
                                           const TwiddleCache &tc, int row0) {
  constexpr int R = StageRadix<N, Ns>::value;
  constexpr bool FIRST = Ns == 1, LAST = Ns * R == N;
  constexpr int NB = V * (N / R);  // butterflies of the stage
  constexpr int Q = (NB + kFftThreads - 1) / kFftThreads;
  const int tid = threadIdx.x;
  float2 v[Q][R];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int flat = tid + q * kFftThreads;
    if (flat < NB) {
      const int rr = flat / (N / R), j = flat % (N / R);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int n = j + r * (N / R);
        if constexpr (FIRST)
          v[q][r] = load_in<INV>(a, in, row0 + rr, n);
        else
          v[q][r] = sm[sidx<N>(rr, n)];
      }
    }
  }
  if constexpr (!FIRST) __syncthreads();  // every read of this stage is done
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int flat = tid + q * kFftThreads;
    if (flat < NB) {
      const int rr = flat / (N / R), j = flat % (N / R);
      const int k = j % Ns;
      if constexpr (!FIRST) twiddle<R>(v[q], tc.w[S][q]);
      dft<R, INV>(v[q]);
      const int d = (j / Ns) * Ns * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int n = d + r * Ns;
        if constexpr (LAST)
          store_out<INV>(a, out, row0 + rr, n, v[q][r]);
        else
          sm[sidx<N>(rr, n)] = v[q][r];
      }
    }
  }
  if constexpr (!LAST) {
    __syncthreads();
    run_stages<N, V, Ns * R, S + 1, INV>(a, in, out, sm, tc, row0);
  }
}

template <int N, int V, bool INV>
__global__ void __launch_bounds__(kFftThreads, 4) fft_row_kernel(const FftArgs a,
                                                              const float2 *__restrict__ in,
                                                              float2 *__restrict__ out) {
  extern __shared__ float2 fft_sm[];
  TwiddleCache tc;
  load_twiddles<N, V, 1, 0, INV>(tc, static_cast<const float2 *>(a.tw_u));
  run_stages<N, V, 1, 0, INV>(a, in, out, fft_sm, tc, int(blockIdx.x) * V);
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
  fn<<<(a.Ny + V - 1) / V, kFftThreads, smem, s>>>(a, static_cast<const float2 *>(in),
                                                   static_cast<float2 *>(out));
  return cudaGetLastError();
}

template <bool INV>
cudaError_t launch_n(const FftArgs &a, const void *in, void *out, cudaStream_t s) {
  if (a.Ny == 0) return cudaSuccess;
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

}  // namespace pg
