#include "gridding_kernels.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <stdexcept>

namespace pg {
namespace {
constexpr double kPi = 3.14159265358979323846;

double bessel_i0(double x) { return std::cyl_bessel_i(0.0, x); }

// Schwab's rational approximation of the J = 6 PSWF (kernels.cc:71-105): a
// polynomial of degree 4 over one of degree 2 in eta^2 - eta_b^2, with
// eta_b = 0.75 on |eta| <= 0.75 and eta_b = 1 on 0.75 < |eta| <= 1.
double pswf_rational(double eta) {
  static const double num_inner[5] = {8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1,
                                      2.312756e-1};
  static const double num_outer[5] = {4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1,
                                      6.412774e-2};
  static const double den_inner[3] = {1., 8.212018e-1, 2.078043e-1};
  static const double den_outer[3] = {1., 9.599102e-1, 2.918724e-1};
  const double a = std::abs(eta);
  const double *nc, *dc;
  double z;
  if (a <= 0.75) {
    nc = num_inner;
    dc = den_inner;
    z = eta * eta - 0.5625;
  } else if (a <= 1.0) {
    nc = num_outer;
    dc = den_outer;
    z = eta * eta - 1.0;
  } else {
    return 0.0;
  }
  // The reference carries a zero sixth numerator coefficient; Horner from the
  // highest non-zero one gives the same value.
  double n = 0.0;
  for (int k = 4; k >= 0; --k) n = n * z + nc[k];
  double d = 0.0;
  for (int k = 2; k >= 0; --k) d = d * z + dc[k];
  return n / d;
}
}  // namespace

GriddingKernel::GriddingKernel(int id, int J, double os) : id_(id), J_(J), os_(os) {
  alpha_ = 2.34 * J;  // Fessler et al. 2003 (kernels.cc:11)
  if (id == kKBMin)   // kernels.cc:259-262
    alpha_ = kPi * std::sqrt(double(J) * J / (os * os) * (os - 0.5) * (os - 0.5) - 0.8);
  sigma_ = (id == kGaussAlt) ? 1.0 : 0.31 * std::pow(double(J), 0.52);  // kernels.cc:56, 307
}

double GriddingKernel::value(double x) const {
  switch (id_) {
    case kKB:
    case kKBMin: {
      const double a = 2 * x / J_;
      return bessel_i0(alpha_ * std::sqrt(1 - a * a)) / bessel_i0(alpha_);
    }
    case kGauss:
    case kGaussAlt: {
      const double a = x / sigma_;
      return std::exp(-0.5 * a * a);
    }
    case kBox:
      return 1.0 / J_;
    case kPSWF: {
      if (J_ != 6) return 0.0;
      const double eta = 2 * x / J_;
      return pswf_rational(eta) * (1 - eta * eta);
    }
  }
  throw std::runtime_error("unknown kernel");
}

double GriddingKernel::correction(double x) const {
  switch (id_) {
    case kKB:
    case kKBMin: {
      // sin(eta)/eta with eta = sqrt((pi x J)^2 - alpha^2), complex when the
      // radicand is negative; the 38828.11016883 scale is the reference's.
      const double r = (kPi * x * J_) * (kPi * x * J_) - alpha_ * alpha_;
      const std::complex<double> eta = std::sqrt(std::complex<double>(r, 0.0));
      return std::real(std::sin(eta) / eta) / 38828.11016883;
    }
    case kGauss:
    case kGaussAlt: {
      const double a = x * sigma_ * kPi;
      return std::sqrt(kPi / 2) / sigma_ * std::exp(-2 * a * a);
    }
    case kBox: {
      const double z = J_ * x * kPi;
      return z == 0.0 ? 1.0 : std::sin(z) / z;
    }
    case kPSWF:
      return (J_ == 6) ? pswf_rational(2 * x) : 0.0;
  }
  throw std::runtime_error("unknown kernel");
}

std::string check_kernel_request(int id, int Ju, int Jv) {
  if (id < kKB || id > kGaussAlt) return "Did not choose valid kernel.";
  if (id == kPSWF && (Ju != 6 || Jv != 6)) return "Incorrect input: PSWF requires a support of 6";
  return "";
}

AxisFit fit_axis(const GriddingKernel &kernel, int taps, int ncoef) {
  const int n = ncoef;
  const double half = 0.5 * taps;
  // Chebyshev nodes of the first kind on [-1, 1].
  std::vector<double> node(n);
  for (int k = 0; k < n; ++k) node[k] = std::cos(kPi * (k + 0.5) / n);

  auto fit_with = [&](int nsub, AxisFit &out) {
    out.ncoef = n;
    out.nsub = nsub;
    out.coef.assign(size_t(taps) * nsub * n, 0.0);
    out.max_error = 0.0;
    std::vector<double> cheb(n), mono(n), tk(n), tkm1(n), tkm2(n);
    for (int j = 0; j < taps; ++j) {
      const double sign = (j & 1) ? -1.0 : 1.0;
      for (int s = 0; s < nsub; ++s) {
        // t in [s/nsub, (s+1)/nsub) maps to x = 2 (t nsub - s) - 1.
        auto f = [&](double x) {
          const double t = (s + 0.5 * (x + 1.0)) / nsub;
          return sign * kernel.value(t + half - 1.0 - j);
        };
        // Chebyshev coefficients from values at the nodes (discrete
        // orthogonality of T_k on the first-kind nodes).
        std::vector<double> fv(n);
        for (int k = 0; k < n; ++k) fv[k] = f(node[k]);
        for (int m = 0; m < n; ++m) {
          double acc = 0.0;
          for (int k = 0; k < n; ++k) acc += fv[k] * std::cos(kPi * m * (k + 0.5) / n);
          cheb[m] = acc * (m == 0 ? 1.0 : 2.0) / n;
        }
        // Monomial coefficients: accumulate c_m T_m(x) with T_m built by the
        // three-term recurrence on coefficient vectors.
        std::fill(mono.begin(), mono.end(), 0.0);
        std::fill(tkm2.begin(), tkm2.end(), 0.0);
        std::fill(tkm1.begin(), tkm1.end(), 0.0);
        tkm2[0] = 1.0;  // T_0
        if (n > 1) tkm1[1] = 1.0;  // T_1
        for (int k = 0; k < n; ++k) mono[k] += cheb[0] * tkm2[k];
        if (n > 1)
          for (int k = 0; k < n; ++k) mono[k] += cheb[1] * tkm1[k];
        for (int m = 2; m < n; ++m) {
          std::fill(tk.begin(), tk.end(), 0.0);
          for (int k = 0; k + 1 < n; ++k) tk[k + 1] += 2.0 * tkm1[k];
          for (int k = 0; k < n; ++k) tk[k] -= tkm2[k];
          for (int k = 0; k < n; ++k) mono[k] += cheb[m] * tk[k];
          tkm2.swap(tkm1);
          tkm1.swap(tk);
        }
        double *dst = &out.coef[(size_t(j) * nsub + s) * n];
        for (int k = 0; k < n; ++k) dst[k] = mono[k];
        // Deviation on a dense grid strictly inside the sub-segment (the
        // end points may sit on a branch point of a piecewise kernel).
        for (int q = 0; q < 256; ++q) {
          const double x = -1.0 + 2.0 * (q + 0.5) / 256.0;
          double p = 0.0;
          for (int k = n - 1; k >= 0; --k) p = p * x + dst[k];
          out.max_error = std::max(out.max_error, std::abs(p - f(x)));
        }
      }
    }
  };

  // Fewest sub-segments that meet the target; a kernel that changes quickly
  // over one tap (narrow supports, the branch point of the PSWF) gets 2 or 4.
  // FP32: the rounding of an FP32 Horner chain is ~1e-7 of the peak already.
  const double target = ncoef >= kCoefF64 ? 1e-13 : 1.5e-7;
  AxisFit best;
  for (int nsub = 1; nsub <= kMaxSub; nsub *= 2) {
    AxisFit fit;
    fit_with(nsub, fit);
    if (nsub == 1 || fit.max_error < best.max_error) best = fit;
    if (best.max_error <= target) break;
  }
  return best;
}

}  // namespace pg
