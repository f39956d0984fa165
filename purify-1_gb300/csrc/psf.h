// Convolution with the point-spread function as an approximation of
// Phi^H Phi (operators::init_psf_convolve_2d, cpp/purify/compact_operators.h:
// 279-307): psf = Phi^H Phi delta at pixel (floor(Ny/2) - 1, floor(Nx/2) - 1);
// A x = F^-1 (F psf * F x) with the unitary image-size FFT F (circular
// convolution, no padding); the operator is A / ||A|| ^ 2 with ||A|| from the
// power method on A, started from a fixed pseudo-random image.
#pragma once
#include <cuda_runtime_api.h>

#include <cstdint>
#include <memory>

#include "operator.h"

namespace pg {

class PsfConvolve {
 public:
  // Builds the PSF with `op` (which must be alive for the call only) and
  // normalises by `power_iters` power-method rounds (0: norm 1).
  static std::unique_ptr<PsfConvolve> create(Operator &op, int power_iters, double power_tol);
  virtual ~PsfConvolve() = default;
  // out = A x / ||A||^2 on device buffers of the operator's precision
  // (imsizey * imsizex values); ordered after `stream`.
  virtual void apply(const void *x, void *out, cudaStream_t stream) = 0;
  virtual double norm() const = 0;
  virtual int64_t device_bytes() const = 0;
};

}  // namespace pg
