// Error paths of the C++ face (include/purify_gb300.hpp) that fail before
// any device work, so they run on a host without a GPU.  Each case must throw
// std::runtime_error, as the reference does on size mismatches
// (cpp/purify/operators.cc:18-20, 63-71).  Prints one line per case:
// "<name> threw" or "<name> did not throw"; exits 0 only if every case threw.
#include <complex>
#include <cstdio>
#include <functional>
#include <stdexcept>
#include <vector>

#include "purify_gb300.hpp"

using Vec = std::vector<std::complex<double>>;
using Real = std::vector<double>;
namespace mo = purify::gb300::measurementoperator;

static bool throws(const char *name, const std::function<void()> &f) {
  bool threw = false;
  try {
    f();
  } catch (const std::runtime_error &) {
    threw = true;
  }
  std::printf("%s %s\n", name, threw ? "threw" : "did not throw");
  return threw;
}

int main() {
  const Real u(10, 0.5), v(10, -0.5), v_short(9, 0.0), w_short(7, 0.0), none;
  const Vec weights_short(9, {1.0, 0.0}), no_weights;
  bool ok = true;
  ok &= throws("uv_size", [&] { mo::init_degrid_operator_2d<Vec>(u, v_short, none, no_weights, 16, 16); });
  ok &= throws("weights_size", [&] {
    mo::init_degrid_operator_2d<Vec>(u, v, none, weights_short, 16, 16);
  });
  ok &= throws("w_size_with_w_term", [&] {
    mo::init_degrid_operator_2d<Vec>(u, v, w_short, no_weights, 16, 16, 2.0, 0, 1e-4,
                                     purify::gb300::kernel::kb, 4, 4, true, 6);
  });
  ok &= throws("w_missing_with_w_term", [&] {
    mo::init_degrid_operator_2d<Vec>(u, v, none, no_weights, 16, 16, 2.0, 0, 1e-4,
                                     purify::gb300::kernel::kb, 4, 4, true, 6);
  });
  purify::gb300::measurementoperator::vis_params<Real, Vec> bad_units;
  bad_units.u = u;
  bad_units.v = v;
  bad_units.units = static_cast<mo::vis_units>(7);
  ok &= throws("unknown_units", [&] { mo::init_degrid_operator_2d<Vec>(bad_units, 16, 16, 1.0, 1.0); });
  purify::gb300::measurementoperator::vis_params<Real, Vec> short_v;
  short_v.u = u;
  short_v.v = v_short;
  short_v.units = mo::vis_units::pixels;
  ok &= throws("vis_params_uv_size", [&] { mo::init_degrid_operator_2d<Vec>(short_v, 16, 16, 1.0, 1.0); });
  return ok ? 0 : 1;
}
