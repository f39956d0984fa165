// Drives the C++ face (include/purify_gb300.hpp) the way a PURIFY caller
// would: build the operator with init_degrid_operator_2d<Vector>, apply
// *op * x and op->adjoint() * y.  Reads u, v, x, y from argv[1] (binary:
// int64 M, int64 n, then u[M], v[M], x[2 n n], y[2 M] as doubles) and writes
// norm, Phi x and Phi^H y to argv[2].
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <vector>

#include "purify_gb300.hpp"

using Vec = std::vector<std::complex<double>>;

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  std::ifstream in(argv[1], std::ios::binary);
  int64_t M = 0, n = 0;
  in.read(reinterpret_cast<char *>(&M), 8);
  in.read(reinterpret_cast<char *>(&n), 8);
  std::vector<double> u(M), v(M), w;
  Vec x(n * n), y(M), weights;
  in.read(reinterpret_cast<char *>(u.data()), 8 * M);
  in.read(reinterpret_cast<char *>(v.data()), 8 * M);
  in.read(reinterpret_cast<char *>(x.data()), 16 * n * n);
  in.read(reinterpret_cast<char *>(y.data()), 16 * M);
  try {
    const auto op = purify::gb300::measurementoperator::init_degrid_operator_2d<Vec>(
        u, v, w, weights, uint32_t(n), uint32_t(n), 2.0, 50, 1e-4,
        purify::gb300::kernel::kb, 4, 4, false, 6, 1.0, 1.0, purify::gb300::precision::fp64);
    const Vec fx = *op * x;
    const Vec ay = op->adjoint() * y;
    // a size mismatch is a std::runtime_error, as in the reference
    bool threw = false;
    try {
      Vec bad(3);
      const Vec r = *op * bad;
    } catch (const std::runtime_error &) {
      threw = true;
    }
    // the vis_params overload: pixels pass unchanged (bit-identical operator),
    // radians go through uv_scale (operators.h:405-410)
    namespace mo = purify::gb300::measurementoperator;
    mo::vis_params<std::vector<double>, Vec> px;
    px.u = u;
    px.v = v;
    px.units = mo::vis_units::pixels;
    const auto op_px = mo::init_degrid_operator_2d<Vec>(px, uint32_t(n), uint32_t(n), 1.0, 1.0,
                                                         2.0, 50, 1e-4, purify::gb300::kernel::kb,
                                                         4, 4, false, 6,
                                                         purify::gb300::precision::fp64);
    mo::vis_params<std::vector<double>, Vec> rad = px;
    const double two_pi = 6.283185307179586;
    for (int64_t m = 0; m < M; ++m) {
      rad.u[m] = u[m] * two_pi / double(2 * n);
      rad.v[m] = v[m] * two_pi / double(2 * n);
    }
    rad.units = mo::vis_units::radians;
    const auto op_rad = mo::init_degrid_operator_2d<Vec>(rad, uint32_t(n), uint32_t(n), 1.0, 1.0,
                                                          2.0, 50, 1e-4, purify::gb300::kernel::kb,
                                                          4, 4, false, 6,
                                                          purify::gb300::precision::fp64);
    const Vec fx_px = *op_px * x, fx_rad = *op_rad * x;
    double e_px = 0, e_rad = 0, nrm = 0;
    for (int64_t m = 0; m < M; ++m) {
      e_px += std::norm(fx_px[m] - fx[m]);
      e_rad += std::norm(fx_rad[m] - fx[m]);
      nrm += std::norm(fx[m]);
    }
    std::printf("units pixels %.3e radians %.3e\n", std::sqrt(e_px / nrm), std::sqrt(e_rad / nrm));
    if (e_px != 0 || !(std::sqrt(e_rad / nrm) < 1e-10)) return 4;
    std::ofstream out(argv[2], std::ios::binary);
    const double norm = 0.0;
    out.write(reinterpret_cast<const char *>(&norm), 8);
    out.write(reinterpret_cast<const char *>(fx.data()), 16 * fx.size());
    out.write(reinterpret_cast<const char *>(ay.data()), 16 * ay.size());
    std::printf("ok threw=%d\n", threw ? 1 : 0);
    return threw ? 0 : 3;
  } catch (const std::exception &e) {
    std::printf("error: %s\n", e.what());
    return 1;
  }
}
