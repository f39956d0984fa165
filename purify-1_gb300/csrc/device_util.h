// Host helpers shared by the operator and batch runtimes: checked cuFFT
// calls, owned device allocations, device selection, and per-precision cuFFT
// dispatch.
#pragma once
#include <cuda_runtime_api.h>
#include <cufft.h>

#include <cstdint>
#include <string>

#include "operator.h"

namespace pg {

inline void cufft_check(cufftResult r, const char *what) {
  if (r == CUFFT_SUCCESS) return;
  if (r == CUFFT_ALLOC_FAILED) throw Error(kOutOfMemory, std::string(what) + ": cuFFT alloc failed");
  throw Error(kCudaError, std::string(what) + ": cuFFT error " + std::to_string(int(r)));
}

// Device allocation owned by an operator or batch.
class DeviceBuffer {
 public:
  DeviceBuffer() = default;
  DeviceBuffer(const DeviceBuffer &) = delete;
  DeviceBuffer &operator=(const DeviceBuffer &) = delete;
  ~DeviceBuffer() {
    if (p_) cudaFree(p_);
  }
  void alloc(size_t bytes, int64_t *counter) {
    if (bytes == 0) bytes = 16;
    cuda_check(cudaMalloc(&p_, bytes), "cudaMalloc");
    bytes_ = bytes;
    if (counter) *counter += int64_t(bytes);
  }
  void upload(const void *src, size_t bytes, cudaStream_t s) {
    if (bytes) cuda_check(cudaMemcpyAsync(p_, src, bytes, cudaMemcpyHostToDevice, s), "upload");
  }
  template <typename T>
  T *as() const {
    return static_cast<T *>(p_);
  }
  void *get() const { return p_; }
  size_t bytes() const { return bytes_; }

 private:
  void *p_ = nullptr;
  size_t bytes_ = 0;
};

class DeviceGuard {
 public:
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev_);
    if (prev_ != dev) cuda_check(cudaSetDevice(dev), "cudaSetDevice");
    dev_ = dev;
  }
  ~DeviceGuard() {
    if (prev_ != dev_) cudaSetDevice(prev_);
  }

 private:
  int prev_ = 0, dev_ = 0;
};

template <typename real>
struct Traits;
template <>
struct Traits<float> {
  static constexpr cufftType kType = CUFFT_C2C;
  static cufftResult exec(cufftHandle h, void *in, void *out, int dir) {
    return cufftExecC2C(h, static_cast<cufftComplex *>(in), static_cast<cufftComplex *>(out), dir);
  }
};
template <>
struct Traits<double> {
  static constexpr cufftType kType = CUFFT_Z2Z;
  static cufftResult exec(cufftHandle h, void *in, void *out, int dir) {
    return cufftExecZ2Z(h, static_cast<cufftDoubleComplex *>(in),
                        static_cast<cufftDoubleComplex *>(out), dir);
  }
};

// cuFFT plan of the Nu columns of an Nv x Nu row-major grid (length Nv,
// stride Nu, one column after the other), bound to `s`; its work area is
// added to *bytes.
template <typename real>
inline cufftHandle make_column_plan(int Nu, int Nv, cudaStream_t s, int64_t *bytes) {
  cufftHandle h = 0;
  int n[1] = {Nv}, embed[1] = {Nv};
  cufft_check(cufftPlanMany(&h, 1, n, embed, Nu, 1, embed, Nu, 1, Traits<real>::kType, Nu),
              "cufftPlanMany");
  const cufftResult r = cufftSetStream(h, s);
  if (r != CUFFT_SUCCESS) {
    cufftDestroy(h);
    cufft_check(r, "cufftSetStream");
  }
  size_t ws = 0;
  if (bytes && cufftGetSize(h, &ws) == CUFFT_SUCCESS) *bytes += int64_t(ws);
  return h;
}


}  // namespace pg
