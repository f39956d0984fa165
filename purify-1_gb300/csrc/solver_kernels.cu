// Element-wise kernels of the forward-backward solver (solver.h).
#include <cuda_runtime.h>

#include "cplx_ops.cuh"
#include "device_kernels.h"
#include "solver.h"

namespace pg {
namespace {
using namespace dev;

// x <- prox(x - step (nx - b)): soft thresholding of the magnitude by
// step * gamma (the proximal map of step * gamma ||.||_1 for complex
// values), then the real and positivity constraints.
template <typename real>
__global__ void fb_step_kernel(cplx<real> *__restrict__ x, const cplx<real> *__restrict__ nx,
                               const cplx<real> *__restrict__ b, int64_t n, real step,
                               const double *__restrict__ gamma, bool real_c, bool pos_c) {
  const real thr = real(double(step) * *gamma);
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x) {
    const cplx<real> xv = x[k], g = nx[k], bv = b[k];
    real vr = xv.x - step * (g.x - bv.x), vi = xv.y - step * (g.y - bv.y);
    if (real_c) vi = real(0);
    const real mag = sqrt(vr * vr + vi * vi);
    const real s = mag > thr ? (mag - thr) / mag : real(0);
    vr *= s;
    vi *= s;
    if (pos_c && vr < real(0)) vr = real(0);
    x[k] = cplx<real>{vr, vi};
  }
}

// Two-stage max with a fixed reduction shape (max is exact in any order).
template <typename real>
__global__ void max_abs_partial(const cplx<real> *__restrict__ x, int64_t n, bool real_part,
                                double *__restrict__ partial) {
  __shared__ double red[256];
  double m = 0;
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n;
       k += int64_t(gridDim.x) * blockDim.x) {
    const cplx<real> v = x[k];
    const double a = real_part ? fabs(double(v.x)) : sqrt(double(v.x) * v.x + double(v.y) * v.y);
    m = a > m ? a : m;
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}
__global__ void max_final(const double *__restrict__ partial, int n, double *__restrict__ out) {
  __shared__ double red[512];
  red[threadIdx.x] = threadIdx.x < n ? partial[threadIdx.x] : 0.0;
  __syncthreads();
  for (int w = 256; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// init: gamma = scale * mx.  Otherwise gamma' = scale * mx replaces gamma
// when |gamma - gamma'| > tol and the update is enabled (update_factory.h:
// 46-54).  The gamma in force is appended to the history.
__global__ void gamma_kernel(double *gamma, const double *mx, double scale, double tol,
                             int enabled, int init, double *history) {
  const double g = scale * *mx;
  if (init)
    *gamma = g;
  else if (enabled && fabs(*gamma - g) > tol)
    *gamma = g;
  if (history) *history = *gamma;
}

int blocks_for(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return int(b < 1 ? 1 : (b > 152 * 16 ? 152 * 16 : b));
}
}  // namespace

template <typename real>
cudaError_t launch_fb_step(void *x, const void *nx, const void *b, int64_t n, double step,
                           const double *gamma, bool real_c, bool pos_c, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  fb_step_kernel<real><<<blocks_for(n), 256, 0, s>>>(
      static_cast<cplx<real> *>(x), static_cast<const cplx<real> *>(nx),
      static_cast<const cplx<real> *>(b), n, real(step), gamma, real_c, pos_c);
  return cudaGetLastError();
}
template <typename real>
cudaError_t launch_max_abs(const void *x, int64_t n, bool real_part, double *partial, double *out,
                           cudaStream_t s) {
  max_abs_partial<real><<<kNormBlocks, 256, 0, s>>>(static_cast<const cplx<real> *>(x), n,
                                                    real_part, partial);
  max_final<<<1, kNormBlocks, 0, s>>>(partial, kNormBlocks, out);
  return cudaGetLastError();
}
cudaError_t launch_gamma_update(double *gamma, const double *mx, double scale, double tol,
                                int enabled, int init, double *history, cudaStream_t s) {
  gamma_kernel<<<1, 1, 0, s>>>(gamma, mx, scale, tol, enabled, init, history);
  return cudaGetLastError();
}

template cudaError_t launch_fb_step<float>(void *, const void *, const void *, int64_t, double,
                                           const double *, bool, bool, cudaStream_t);
template cudaError_t launch_fb_step<double>(void *, const void *, const void *, int64_t, double,
                                            const double *, bool, bool, cudaStream_t);
template cudaError_t launch_max_abs<float>(const void *, int64_t, bool, double *, double *,
                                           cudaStream_t);
template cudaError_t launch_max_abs<double>(const void *, int64_t, bool, double *, double *,
                                            cudaStream_t);

}  // namespace pg
