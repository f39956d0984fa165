// FP64 gridding-kernel family and its piecewise-polynomial fit (host side).
#pragma once
#include <algorithm>
#include <cmath>
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

// The J tap weights at t in [0, 1), evaluated in `real` arithmetic exactly as
// the device does it (tap_weights in device_kernels.cu): one Horner chain per
// sub-segment when nsub > 1, else an even/odd split shared by mirrored taps.
template <typename real>
void eval_taps(const AxisFit &fit, int J, double t_in, real *k) {
  const int nc = fit.ncoef;
  const real t = real(t_in);
  auto c = [&](int j, int s, int q) { return real(fit.coef[(size_t(j) * fit.nsub + s) * nc + q]); };
  if (fit.nsub > 1) {
    const real ts = t * real(fit.nsub);
    const int s = std::min(int(ts), fit.nsub - 1);
    const real x = real(2) * (ts - real(s)) - real(1);
    for (int j = 0; j < J; ++j) {
      real acc = c(j, s, nc - 1);
      for (int q = nc - 2; q >= 0; --q) acc = std::fma(acc, x, c(j, s, q));
      k[j] = acc;
    }
    return;
  }
  const real x = real(2) * t - real(1);
  const real x2 = x * x;
  const int ne = (nc + 1) / 2, no = nc / 2;
  for (int j = 0; j < (J + 1) / 2; ++j) {
    real e = c(j, 0, 2 * (ne - 1));
    for (int q = ne - 2; q >= 0; --q) e = std::fma(e, x2, c(j, 0, 2 * q));
    real o = c(j, 0, 2 * no - 1);
    for (int q = no - 2; q >= 0; --q) o = std::fma(o, x2, c(j, 0, 2 * q + 1));
    k[j] = std::fma(x, o, e);
    if (J - 1 - j != j) {
      const real mirror = std::fma(-x, o, e);
      k[J - 1 - j] = (J % 2 == 1) ? mirror : -mirror;
    }
  }
}

}  // namespace pg
