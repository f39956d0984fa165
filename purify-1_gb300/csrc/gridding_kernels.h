// FP64 gridding-kernel family and its piecewise-polynomial fit (host side).
#pragma once
#include <string>
#include <vector>

#include "pg_types.h"

namespace pg {

// One separable gridding kernel of the reference's family
// (cpp/purify/kernels.cc:7-230, bound by create_kernels kernels.cc:233-323).
// value(x) is the spatial kernel on the support |x| <= J/2; correction(x) is
// its Fourier transform evaluated at the already-shifted argument that
// create_kernels passes (pixel / ftsize - 0.5).
class GriddingKernel {
 public:
  GriddingKernel(int id, int J, double oversample_ratio);
  double value(double x) const;
  double correction(double x) const;
  int id() const { return id_; }
  int support() const { return J_; }

 private:
  int id_, J_;
  double os_, alpha_, sigma_;
};

// Validates a kernel request the way create_kernels does; returns an empty
// string when it is accepted, else the reason.
std::string check_kernel_request(int id, int Ju, int Jv);

// Result of fitting one axis: coefficients laid out [tap][sub][coef], the
// number of sub-segments per tap, and the largest deviation from value()
// found on a dense check grid (absolute, kernel peak is O(1)).
struct AxisFit {
  std::vector<double> coef;
  int ncoef = 0;
  int nsub = 1;
  double max_error = 0;
};

// Fits P_{j,s} (see PolyAxis) for taps j = 0..taps-1 of `kernel` by Chebyshev
// interpolation in FP64, converted to the monomial basis on [-1, 1].
AxisFit fit_axis(const GriddingKernel &kernel, int taps, int ncoef);

}  // namespace pg
