#include "ingest.h"

#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <string>

#include "device_util.h"
#include "ingest_kernels.h"
#include "operator.h"

namespace pg {

int64_t vis_file_rows(const std::string &path) {
  std::ifstream f(path);
  if (!f) throw Error(kInvalidArgument, "cannot open visibility file " + path);
  int64_t rows = 0;
  std::string line;
  while (std::getline(f, line)) ++rows;
  return rows;
}

namespace {
// One white-space separated real; nan and inf are accepted (utilities.cc:133-138).
double next_real(std::ifstream &f, const std::string &path, int64_t row) {
  std::string tok;
  if (!(f >> tok))
    throw Error(kInvalidArgument, path + ": row " + std::to_string(row) + " is short");
  const char *s = tok.c_str();
  char *end = nullptr;
  errno = 0;
  const double x = std::strtod(s, &end);
  if (end == s || *end != '\0')
    throw Error(kInvalidArgument, path + ": row " + std::to_string(row) + ": '" + tok +
                                      "' is not a number");
  return x;
}
}  // namespace

void read_visibility(const std::string &path, bool w_term, int64_t rows, double *u, double *v,
                     double *w, std::complex<double> *vis, std::complex<double> *weights) {
  std::ifstream f(path);
  if (!f) throw Error(kInvalidArgument, "cannot open visibility file " + path);
  for (int64_t r = 0; r < rows; ++r) {
    const double uu = next_real(f, path, r), vv = next_real(f, path, r);
    const double ww = w_term ? next_real(f, path, r) : 0.0;
    const double re = next_real(f, path, r), im = next_real(f, path, r);
    const double sigma = next_real(f, path, r);
    u[r] = uu;
    v[r] = -vv;  // the reflection of utilities.cc:178
    if (w) w[r] = ww;
    vis[r] = std::complex<double>(re, im);
    weights[r] = std::complex<double>(1.0 / sigma, 0.0);
  }
}

void init_weights(const double *u, const double *v, const std::complex<double> *weights,
                  int64_t M, double oversample_factor, int weighting, double R, int ftsizeu,
                  int ftsizev, int device, std::complex<double> *out) {
  if (M < 0) throw Error(kInvalidArgument, "negative number of visibilities");
  switch (weighting) {
    case kWeightNone:
      for (int64_t i = 0; i < M; ++i) out[i] = 1.0;
      return;
    case kWeightNatural:
    case kWeightWhiten:
      for (int64_t i = 0; i < M; ++i) out[i] = weights[i];
      return;
    case kWeightUniform:
    case kWeightRobust:
      break;
    default:
      throw Error(kInvalidArgument, "Wrong weighting type, " + std::to_string(weighting) +
                                        " not recognised.");
  }
  if (ftsizeu < 1 || ftsizev < 1) throw Error(kInvalidArgument, "empty grid");
  if (!(oversample_factor > 0)) throw Error(kInvalidArgument, "oversample_factor must be > 0");
  for (int64_t i = 0; i < M; ++i)
    if (!std::isfinite(u[i]) || !std::isfinite(v[i]))
      throw Error(kInvalidArgument, "visibility " + std::to_string(i) +
                                        " has a non-finite u or v coordinate");
  if (M == 0) return;
  DeviceGuard guard(device);
  cudaStream_t s = nullptr;
  cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
  try {
    DeviceBuffer du, dv, dw, dout, counts, sums;
    du.alloc(sizeof(double) * M, nullptr);
    dv.alloc(sizeof(double) * M, nullptr);
    dw.alloc(16 * size_t(M), nullptr);
    dout.alloc(16 * size_t(M), nullptr);
    counts.alloc(sizeof(uint32_t) * size_t(ftsizeu) * ftsizev, nullptr);
    sums.alloc(sizeof(double) * (4 + 4 * kIngestBlocks) + sizeof(unsigned long long), nullptr);
    du.upload(u, sizeof(double) * M, s);
    dv.upload(v, sizeof(double) * M, s);
    dw.upload(weights, 16 * size_t(M), s);
    cuda_check(cudaMemsetAsync(counts.get(), 0, sizeof(uint32_t) * size_t(ftsizeu) * ftsizev, s),
               "cudaMemsetAsync");
    cuda_check(launch_weights_histogram(du.as<double>(), dv.as<double>(), M, 1.0 / oversample_factor,
                                        ftsizeu, ftsizev, counts.as<uint32_t>(), s),
               "histogram");
    cuda_check(launch_weights_sums(dw.as<double>(), M, counts.as<uint32_t>(),
                                   int64_t(ftsizeu) * ftsizev, sums.as<double>(), s),
               "sums");
    double hsums[4];
    cuda_check(cudaMemcpyAsync(hsums, sums.get(), sizeof(hsums), cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaStreamSynchronize(s), "init_weights");
    // sum_weights = sum w^2 (complex), sum_grid_weights2 = sum count^2,
    // robust_scale = sum_weights / sum_grid_weights2 * 25 * 10^(-2R)
    const std::complex<double> sum_weights(hsums[0], hsums[1]);
    const double sum_grid2 = hsums[2];
    const std::complex<double> robust_scale =
        sum_weights / sum_grid2 * 25. * std::pow(10., -2 * R);
    cuda_check(launch_weights_apply(du.as<double>(), dv.as<double>(), dw.as<double>(), M,
                                    1.0 / oversample_factor, ftsizeu, ftsizev,
                                    counts.as<uint32_t>(), weighting == kWeightRobust,
                                    robust_scale.real(), robust_scale.imag(), dout.as<double>(), s),
               "weights");
    cuda_check(cudaMemcpyAsync(out, dout.get(), 16 * size_t(M), cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaStreamSynchronize(s), "init_weights");
  } catch (...) {
    cudaStreamDestroy(s);
    throw;
  }
  cudaStreamDestroy(s);
}

}  // namespace pg
