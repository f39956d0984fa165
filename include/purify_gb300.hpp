// purify_gb300.hpp — C++ face of the GB300 measurement operator.
//
// Rebuilds the reference's factory signature on top of the C ABI in
// purify_gb300.h:
//
//   purify::gb300::measurementoperator::init_degrid_operator_2d<T>(
//       u, v, w, weights, imsizey, imsizex, oversample_ratio = 2,
//       power_iters = 100, power_tol = 1e-4, kernel = kb, Ju = 4, Jv = 4,
//       w_term = false, Jw = 6, cellx = 1, celly = 1)
//     -> std::shared_ptr<sopt::LinearTransform<T> const>
//
// which replaces measurementoperator::init_degrid_operator_2d
// (cpp/purify/operators.h:372-396) and the vis_params overload
// (operators.h:398-414).  Failures surface as std::runtime_error, the
// reference's error type (operators.cc:18-20, operators.h:187).  Applies take
// and return host complex<double> vectors, as the reference's closures do
// (sopt::OperatorFunction resizes `out` itself, operators.h:159, 172, 244).
//
// T is any vector of std::complex<double> with data(), size() and resize()
// (Eigen's Vector<t_complex>, std::vector<std::complex<double>>).  When the
// real sopt headers are on the include path their LinearTransform is used;
// otherwise a minimal stand-in with the same calling surface is defined here.
#ifndef PURIFY_GB300_HPP
#define PURIFY_GB300_HPP

#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "purify_gb300.h"

#if defined(__has_include)
#if __has_include(<sopt/linear_transform.h>) && __has_include(<Eigen/Core>)
#include <sopt/linear_transform.h>
#define PURIFY_GB300_HAVE_SOPT 1
#endif
#endif

#ifndef PURIFY_GB300_HAVE_SOPT
// Stand-ins for the two sopt types the operator API uses (sopt is absent).
namespace sopt {
template <class T>
using OperatorFunction = std::function<void(T &, const T &)>;

// Same construction and application as sopt::LinearTransform: a direct and
// an indirect function with their {offset, stride, size} descriptors;
// `op * x` applies the direct one, `op.adjoint() * y` the indirect one.
template <class T>
class LinearTransform {
 public:
  LinearTransform(OperatorFunction<T> direct, std::array<std::int64_t, 3> dsizes,
                  OperatorFunction<T> indirect, std::array<std::int64_t, 3> isizes)
      : direct_(std::move(direct)), indirect_(std::move(indirect)), dsizes_(dsizes),
        isizes_(isizes) {}
  T operator*(const T &x) const {
    T out;
    direct_(out, x);
    return out;
  }
  LinearTransform adjoint() const { return LinearTransform(indirect_, isizes_, direct_, dsizes_); }
  const std::array<std::int64_t, 3> &sizes() const { return dsizes_; }
  const std::array<std::int64_t, 3> &adjoint_sizes() const { return isizes_; }

 private:
  OperatorFunction<T> direct_, indirect_;
  std::array<std::int64_t, 3> dsizes_, isizes_;
};
}  // namespace sopt
#endif

namespace purify {
namespace gb300 {

inline void check(int status) {
  if (status != PURIFY_GB300_OK) throw std::runtime_error(purify_gb300_last_error());
}

// Kernel names of kernels::kernel (cpp/purify/kernels.h:15).
enum class kernel { kb = 0, gauss = 1, box = 2, pswf = 3, kbmin = 4, gauss_alt = 5 };
enum class precision { fp32 = PURIFY_GB300_FP32, fp64 = PURIFY_GB300_FP64 };

// Owning handle of a device operator.  Shared by the closures of the
// LinearTransform; applies are ordered inside the library, so concurrent
// calls from several threads are safe.
class Operator {
 public:
  explicit Operator(const purify_gb300_create_args &args) {
    purify_gb300_operator *h = nullptr;
    check(purify_gb300_operator_create(&args, &h));
    h_.reset(h, [](purify_gb300_operator *p) { purify_gb300_operator_destroy(p); });
    check(purify_gb300_operator_info(h_.get(), &info_));
  }
  template <class T>
  void forward(T &out, const T &x) const {
    if (std::int64_t(x.size()) != std::int64_t(info_.imsizex) * info_.imsizey)
      throw std::runtime_error("image vector has the wrong size");
    out.resize(info_.M);
    check(purify_gb300_forward_host(h_.get(), reinterpret_cast<const double *>(x.data()),
                                    reinterpret_cast<double *>(out.data())));
  }
  template <class T>
  void adjoint(T &out, const T &y) const {
    if (std::int64_t(y.size()) != info_.M)
      throw std::runtime_error("visibility vector has the wrong size");
    out.resize(std::int64_t(info_.imsizex) * info_.imsizey);
    check(purify_gb300_adjoint_host(h_.get(), reinterpret_cast<const double *>(y.data()),
                                    reinterpret_cast<double *>(out.data())));
  }
  double norm() const {
    double n = 0;
    check(purify_gb300_get_norm(h_.get(), &n));
    return n;
  }
  const purify_gb300_info &info() const { return info_; }
  purify_gb300_operator *handle() const { return h_.get(); }

 private:
  std::shared_ptr<purify_gb300_operator> h_;
  purify_gb300_info info_{};
};

namespace measurementoperator {

// measurementoperator::init_degrid_operator_2d (operators.h:373-396), u and v
// in grid pixels.  `prec` selects the arithmetic (FP32 computes in
// complex<float> on the device; the interface stays complex<double>).
template <class T, class RealVec, class ComplexVec>
std::shared_ptr<sopt::LinearTransform<T> const> init_degrid_operator_2d(
    const RealVec &u, const RealVec &v, const RealVec &w, const ComplexVec &weights,
    const std::uint32_t &imsizey, const std::uint32_t &imsizex,
    const double &oversample_ratio = 2, const std::uint32_t &power_iters = 100,
    const double &power_tol = 1e-4, const kernel kern = kernel::kb, const std::uint32_t Ju = 4,
    const std::uint32_t Jv = 4, const bool w_term = false, const std::uint32_t Jw = 6,
    const double &cellx = 1, const double &celly = 1, const precision prec = precision::fp32,
    const int device = 0) {
  // Size checks of details::init_gridding_matrix_2d (operators.cc:18-20,
  // 63-71).  An empty weights vector stands for unit weights (the reference
  // needs M of them); any other size is an error, as in the reference.  w is
  // read only with w_term, where it must hold M values; without w_term the
  // reference reads no w either.
  if (u.size() != v.size())
    throw std::runtime_error(
        "Size of u and v vectors are not the same for creating gridding matrix.");
  if (w_term && w.size() != u.size())
    throw std::runtime_error(
        "Size of u and w vectors are not the same for creating gridding matrix.");
  if (weights.size() != 0 && weights.size() != u.size())
    throw std::runtime_error(
        "Size of u and weights vectors are not the same for creating gridding matrix.");
  purify_gb300_create_args a;
  purify_gb300_default_args(&a);
  a.u = u.data();
  a.v = v.data();
  a.w = w_term ? w.data() : nullptr;
  a.weights = weights.size() == u.size() ? reinterpret_cast<const double *>(weights.data())
                                         : nullptr;
  a.M = std::int64_t(u.size());
  a.imsizey = imsizey;
  a.imsizex = imsizex;
  a.oversample_ratio = oversample_ratio;
  a.power_iters = power_iters;
  a.power_tol = power_tol;
  a.kernel = int(kern);
  a.Ju = Ju;
  a.Jv = Jv;
  a.w_term = w_term ? 1 : 0;
  a.Jw = Jw;
  a.cellx = cellx;
  a.celly = celly;
  a.precision = int(prec);
  a.device = device;
  auto op = std::make_shared<const Operator>(a);
  const std::array<std::int64_t, 3> N = {0, 1, std::int64_t(imsizey) * imsizex};
  const std::array<std::int64_t, 3> M = {0, 1, std::int64_t(u.size())};
  sopt::OperatorFunction<T> direct = [op](T &out, const T &x) { op->forward(out, x); };
  sopt::OperatorFunction<T> indirect = [op](T &out, const T &y) { op->adjoint(out, y); };
  return std::make_shared<sopt::LinearTransform<T> const>(direct, M, indirect, N);
}

// The vis_params overload (operators.h:398-414): coordinates in wavelengths
// are converted with set_cell_size + uv_scale (utilities.cc:208-278).
template <class T, class RealVec, class ComplexVec>
std::shared_ptr<sopt::LinearTransform<T> const> init_degrid_operator_2d_lambda(
    const RealVec &u_lambda, const RealVec &v_lambda, const RealVec &w,
    const ComplexVec &weights, const std::uint32_t &imsizey, const std::uint32_t &imsizex,
    const double &cell_x, const double &cell_y, const double &oversample_ratio = 2,
    const std::uint32_t &power_iters = 100, const double &power_tol = 1e-4,
    const kernel kern = kernel::kb, const std::uint32_t Ju = 4, const std::uint32_t Jv = 4,
    const bool w_term = false, const std::uint32_t Jw = 6,
    const precision prec = precision::fp32) {
  std::vector<double> up(u_lambda.size()), vp(v_lambda.size());
  check(purify_gb300_lambda_to_pixels(
      u_lambda.data(), v_lambda.data(), std::int64_t(u_lambda.size()), cell_x, cell_y,
      std::uint32_t(std::floor(oversample_ratio * imsizex)),
      std::uint32_t(std::floor(oversample_ratio * imsizey)), up.data(), vp.data()));
  return init_degrid_operator_2d<T>(up, vp, w, weights, imsizey, imsizex, oversample_ratio,
                                    power_iters, power_tol, kern, Ju, Jv, w_term, Jw, cell_x,
                                    cell_y, prec);
}

// utilities::vis_units and the fields of utilities::vis_params that the
// operator reads (cpp/purify/utilities.h:14-55), for callers without the
// reference's headers.  The overload below accepts any type with these
// fields, the reference's vis_params included (its units enum has the same
// order).
enum class vis_units { lambda = PURIFY_GB300_UNITS_LAMBDA, radians = PURIFY_GB300_UNITS_RADIANS,
                       pixels = PURIFY_GB300_UNITS_PIXELS };
template <class RealVec, class ComplexVec>
struct vis_params {
  RealVec u, v, w;
  ComplexVec weights;
  vis_units units = vis_units::lambda;
};

// The vis_params overload (operators.h:398-414): wavelengths are converted
// by set_cell_size + uv_scale, radians by uv_scale, pixels pass unchanged
// (utilities.cc:208-278); the cell sizes also reach the w-projection rows.
template <class T, class VisParams>
std::shared_ptr<sopt::LinearTransform<T> const> init_degrid_operator_2d(
    const VisParams &uv_vis, const std::uint32_t &imsizey, const std::uint32_t &imsizex,
    const double &cell_x, const double &cell_y, const double &oversample_ratio = 2,
    const std::uint32_t &power_iters = 100, const double &power_tol = 1e-4,
    const kernel kern = kernel::kb, const std::uint32_t Ju = 4, const std::uint32_t Jv = 4,
    const bool w_term = false, const std::uint32_t Jw = 6,
    const precision prec = precision::fp32, const int device = 0) {
  if (uv_vis.u.size() != uv_vis.v.size())
    throw std::runtime_error(
        "Size of u and v vectors are not the same for creating gridding matrix.");
  std::vector<double> up(uv_vis.u.size()), vp(uv_vis.v.size());
  check(purify_gb300_uv_to_pixels(
      uv_vis.u.data(), uv_vis.v.data(), std::int64_t(uv_vis.u.size()),
      static_cast<std::int32_t>(uv_vis.units), cell_x, cell_y,
      std::uint32_t(std::floor(oversample_ratio * imsizex)),
      std::uint32_t(std::floor(oversample_ratio * imsizey)), up.data(), vp.data()));
  return init_degrid_operator_2d<T>(up, vp, uv_vis.w, uv_vis.weights, imsizey, imsizex,
                                    oversample_ratio, power_iters, power_tol, kern, Ju, Jv,
                                    w_term, Jw, cell_x, cell_y, prec, device);
}

}  // namespace measurementoperator
}  // namespace gb300
}  // namespace purify

#endif  // PURIFY_GB300_HPP
