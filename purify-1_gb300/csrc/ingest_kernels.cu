// Visibility-weighting kernels: histogram of visibilities per grid cell,
// deterministic sums, per-visibility weights (utilities::init_weights,
// cpp/purify/utilities.cc:569-608).
#include <cuda_runtime.h>

#include <cstdint>

#include "ingest_kernels.h"

namespace pg {
namespace {

// utilities::mod (utilities.cc:350-357) of an integer-valued x: fmod wrapped
// to [0, y); exact for integers, kept in range defensively.
__device__ __forceinline__ int cell_index(double x, int n) {
  double r = fmod(floor(x), double(n));
  if (r < 0) r += double(n);
  int k = int(r);
  return k >= n ? k - n : k;
}

__global__ void histogram_kernel(const double *__restrict__ u, const double *__restrict__ v,
                                 int64_t M, double scale, int Nu, int Nv,
                                 uint32_t *__restrict__ counts) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < M;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int q = cell_index(u[i] * scale, Nu), p = cell_index(v[i] * scale, Nv);
    atomicAdd(counts + int64_t(p) * Nu + q, 1u);
  }
}

// Block b: FP64 sum of w^2 over i = b * 256 + t + k * stride in ascending k,
// then a fixed tree; integer sum of count^2, exact in any order.
__global__ void sums_partial(const double2 *__restrict__ w, int64_t M,
                             const uint32_t *__restrict__ counts, int64_t ncells,
                             double *__restrict__ partial, unsigned long long *__restrict__ c2) {
  __shared__ double re[256], im[256];
  __shared__ unsigned long long cc[256];
  double sr = 0, si = 0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < M;
       i += int64_t(gridDim.x) * blockDim.x) {
    const double2 z = w[i];
    sr += z.x * z.x - z.y * z.y;
    si += 2.0 * z.x * z.y;
  }
  unsigned long long sc = 0;
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < ncells;
       k += int64_t(gridDim.x) * blockDim.x) {
    const unsigned long long c = counts[k];
    sc += c * c;
  }
  re[threadIdx.x] = sr;
  im[threadIdx.x] = si;
  cc[threadIdx.x] = sc;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      re[threadIdx.x] += re[threadIdx.x + h];
      im[threadIdx.x] += im[threadIdx.x + h];
      cc[threadIdx.x] += cc[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = re[0];
    partial[2 * blockIdx.x + 1] = im[0];
    atomicAdd(c2, cc[0]);
  }
}

__global__ void sums_final(const double *__restrict__ partial, int n,
                           const unsigned long long *__restrict__ c2, double *__restrict__ out) {
  __shared__ double re[kIngestBlocks], im[kIngestBlocks];
  re[threadIdx.x] = threadIdx.x < n ? partial[2 * threadIdx.x] : 0.0;
  im[threadIdx.x] = threadIdx.x < n ? partial[2 * threadIdx.x + 1] : 0.0;
  __syncthreads();
  for (int h = kIngestBlocks / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      re[threadIdx.x] += re[threadIdx.x + h];
      im[threadIdx.x] += im[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = re[0];
    out[1] = im[0];
    out[2] = double(*c2);
    out[3] = 0;
  }
}

// Principal square root of a + bi by the half-angle formulas.
__device__ __forceinline__ double2 csqrt(double a, double b) {
  const double r = hypot(a, b);
  const double t = sqrt(0.5 * (fabs(a) + r));
  if (t == 0) return double2{0, 0};
  return a >= 0 ? double2{t, b / (2 * t)} : double2{fabs(b) / (2 * t), copysign(t, b)};
}

__global__ void apply_kernel(const double *__restrict__ u, const double *__restrict__ v,
                             const double2 *__restrict__ w, int64_t M, double scale, int Nu,
                             int Nv, const uint32_t *__restrict__ counts, bool robust,
                             double rs_re, double rs_im, double2 *__restrict__ out) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < M;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int q = cell_index(u[i] * scale, Nu), p = cell_index(v[i] * scale, Nv);
    const double g = sqrt(double(counts[int64_t(p) * Nu + q]));  // gridded weight
    double2 d;
    if (robust) {
      const double g2 = g * g;
      d = csqrt(1.0 + rs_re * g2, rs_im * g2);
    } else {
      d = double2{g, 0.0};
    }
    const double2 z = w[i];
    const double den = d.x * d.x + d.y * d.y;
    out[i] = double2{(z.x * d.x + z.y * d.y) / den, (z.y * d.x - z.x * d.y) / den};
  }
}

int blocks_for(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return int(b < 1 ? 1 : (b > 152 * 16 ? 152 * 16 : b));
}

}  // namespace

cudaError_t launch_weights_histogram(const double *u, const double *v, int64_t M, double scale,
                                     int Nu, int Nv, uint32_t *counts, cudaStream_t s) {
  if (M == 0) return cudaSuccess;
  histogram_kernel<<<blocks_for(M), 256, 0, s>>>(u, v, M, scale, Nu, Nv, counts);
  return cudaGetLastError();
}

cudaError_t launch_weights_sums(const double *w, int64_t M, const uint32_t *counts,
                                int64_t ncells, double *sums, cudaStream_t s) {
  double *partial = sums + 4;
  unsigned long long *c2 = reinterpret_cast<unsigned long long *>(partial + 2 * kIngestBlocks);
  cudaError_t e = cudaMemsetAsync(c2, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  sums_partial<<<kIngestBlocks, 256, 0, s>>>(reinterpret_cast<const double2 *>(w), M, counts,
                                             ncells, partial, c2);
  sums_final<<<1, kIngestBlocks, 0, s>>>(partial, kIngestBlocks, c2, sums);
  return cudaGetLastError();
}

cudaError_t launch_weights_apply(const double *u, const double *v, const double *w, int64_t M,
                                 double scale, int Nu, int Nv, const uint32_t *counts, bool robust,
                                 double rs_re, double rs_im, double *out, cudaStream_t s) {
  if (M == 0) return cudaSuccess;
  apply_kernel<<<blocks_for(M), 256, 0, s>>>(u, v, reinterpret_cast<const double2 *>(w), M, scale,
                                             Nu, Nv, counts, robust, rs_re, rs_im,
                                             reinterpret_cast<double2 *>(out));
  return cudaGetLastError();
}

}  // namespace pg
