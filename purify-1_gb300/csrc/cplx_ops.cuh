// Complex value types of the device code and component-wise complex
// arithmetic on them.
#pragma once
#include <cuda_runtime.h>

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

// Component-wise complex arithmetic.  For float these are Blackwell's paired
// FP32 instructions (one instruction for both components, each component
// rounded exactly as fmaf / fadd / fmul), for double two scalar operations:
// either way the result is bit-identical to the scalar form.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ double2 fma2(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ double2 add2(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ double2 mul2(double2 a, double2 b) {
  return make_double2(a.x * b.x, a.y * b.y);
}
template <typename real>
__device__ __forceinline__ cplx<real> splat(real k) {
  return cplx<real>{k, k};
}

}  // namespace dev
}  // namespace pg
