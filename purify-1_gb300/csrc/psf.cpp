#include "psf.h"

#include <cufft.h>

#include <cmath>
#include <complex>
#include <mutex>
#include <vector>

#include "device_kernels.h"
#include "device_util.h"

namespace pg {
namespace {

template <typename real>
class PsfT final : public PsfConvolve {
 public:
  PsfT(Operator &op, int power_iters, double power_tol);
  ~PsfT() override;
  void apply(const void *x, void *out, cudaStream_t stream) override;
  double norm() const override { return norm_; }
  int64_t device_bytes() const override { return bytes_; }

 private:
  void apply_raw(const void *x, void *out, double scale);
  int device_ = 0, Nx_ = 0, Ny_ = 0;
  int64_t N_ = 0, bytes_ = 0;
  double norm_ = 1.0;
  DeviceBuffer ft_, tmp_, partial_, sq_;
  cufftHandle fft_ = 0;
  bool fft_ok_ = false;
  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev_in_ = nullptr, ev_out_ = nullptr;
  std::mutex mu_;
};

template <typename real>
PsfT<real>::PsfT(Operator &op, int power_iters, double power_tol) {
  const OperatorInfo info = op.info();
  device_ = info.device;
  DeviceGuard guard(device_);
  Nx_ = int(info.imsizex);
  Ny_ = int(info.imsizey);
  N_ = int64_t(Nx_) * Ny_;
  using C = std::complex<real>;
  cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  cuda_check(cudaEventCreateWithFlags(&ev_in_, cudaEventDisableTiming), "cudaEventCreate");
  cuda_check(cudaEventCreateWithFlags(&ev_out_, cudaEventDisableTiming), "cudaEventCreate");
  ft_.alloc(sizeof(C) * N_, &bytes_);
  tmp_.alloc(sizeof(C) * N_, &bytes_);
  partial_.alloc(sizeof(double) * kNormBlocks, &bytes_);
  sq_.alloc(sizeof(double), &bytes_);
  cufft_check(cufftPlan2d(&fft_, Ny_, Nx_, Traits<real>::kType), "cufftPlan2d");
  fft_ok_ = true;
  cufft_check(cufftSetStream(fft_, stream_), "cufftSetStream");
  // psf = Phi^H Phi delta, delta at sub2ind(floor(Ny/2) - 1, floor(Nx/2) - 1)
  // (utilities.cc:321-333, row * cols + col)
  const int64_t index = int64_t(Ny_ / 2 - 1) * Nx_ + (Nx_ / 2 - 1);
  cuda_check(launch_delta<real>(tmp_.get(), N_, index, stream_), "delta");
  op.normal(tmp_.get(), ft_.get(), stream_);
  // F psf with the unitary scale 1 / sqrt(N)
  cufft_check(Traits<real>::exec(fft_, ft_.get(), ft_.get(), CUFFT_FORWARD), "cufftExec");
  cuda_check(launch_scale<real>(ft_.get(), N_, 1.0 / std::sqrt(double(N_)), stream_), "scale");
  // Power method on A (adjoint = identity): x <- A x, estimate ||A x||,
  // stop when its relative change is below tol^2, norm = sqrt(estimate).
  if (power_iters > 0) {
    // The all-ones image is the zero-frequency eigenvector of a circular
    // convolution, so the iteration starts from a fixed pseudo-random image
    // (the reference starts from a random one): x_k = h(k) / 2^32 - 1/2 with
    // Knuth's multiplicative hash h(k) = 2654435761 k mod 2^32, normalised.
    std::vector<C> x0(N_);
    double nn = 0;
    for (int64_t k = 0; k < N_; ++k) {
      const double r = double(uint32_t(uint64_t(k) * 2654435761ull)) / 4294967296.0 - 0.5;
      x0[k] = C(real(r), real(0));
      nn += r * r;
    }
    const double inv = 1.0 / std::sqrt(nn);
    for (auto &c : x0) c *= real(inv);
    DeviceBuffer x;
    x.alloc(sizeof(C) * N_, nullptr);
    x.upload(x0.data(), sizeof(C) * N_, stream_);
    double old_value = 0;
    for (int i = 0; i < power_iters; ++i) {
      apply_raw(x.get(), x.get(), 1.0);
      cuda_check(launch_sq_norm<real>(x.get(), N_, partial_.as<double>(), sq_.as<double>(),
                                      stream_),
                 "norm");
      double sq = 0;
      cuda_check(cudaMemcpyAsync(&sq, sq_.get(), sizeof(double), cudaMemcpyDeviceToHost, stream_),
                 "D2H");
      cuda_check(cudaStreamSynchronize(stream_), "power_method");
      const double value = std::sqrt(sq);
      if (!(value > 0)) throw Error(kNormNotPositive, "Operator norm is not greater than zero.");
      cuda_check(launch_scale<real>(x.get(), N_, 1.0 / value, stream_), "scale");
      if (power_tol * power_tol > std::abs(old_value - value) / old_value) {
        old_value = value;
        break;
      }
      old_value = value;
    }
    norm_ = std::sqrt(old_value);
  }
  cuda_check(cudaStreamSynchronize(stream_), "psf setup");
}

template <typename real>
PsfT<real>::~PsfT() {
  if (stream_) cudaStreamSynchronize(stream_);
  if (fft_ok_) cufftDestroy(fft_);
  if (ev_in_) cudaEventDestroy(ev_in_);
  if (ev_out_) cudaEventDestroy(ev_out_);
  if (stream_) cudaStreamDestroy(stream_);
}

// out = F^-1 (ft * F x) * scale with the unitary F on both sides: the two
// 1 / sqrt(N) factors are folded into the product, as is `scale`.
template <typename real>
void PsfT<real>::apply_raw(const void *x, void *out, double scale) {
  cufft_check(Traits<real>::exec(fft_, const_cast<void *>(x), tmp_.get(), CUFFT_FORWARD),
              "cufftExec");
  cuda_check(launch_cmul_scale<real>(tmp_.get(), ft_.get(), N_, scale / double(N_), stream_),
             "multiply");
  cufft_check(Traits<real>::exec(fft_, tmp_.get(), out, CUFFT_INVERSE), "cufftExec");
}

template <typename real>
void PsfT<real>::apply(const void *x, void *out, cudaStream_t user) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  cuda_check(cudaEventRecord(ev_in_, user), "cudaEventRecord");
  cuda_check(cudaStreamWaitEvent(stream_, ev_in_, 0), "cudaStreamWaitEvent");
  apply_raw(x, out, 1.0 / (norm_ * norm_));
  cuda_check(cudaEventRecord(ev_out_, stream_), "cudaEventRecord");
  cuda_check(cudaStreamWaitEvent(user, ev_out_, 0), "cudaStreamWaitEvent");
}

}  // namespace

std::unique_ptr<PsfConvolve> PsfConvolve::create(Operator &op, int power_iters, double power_tol) {
  if (op.info().fp64) return std::unique_ptr<PsfConvolve>(new PsfT<double>(op, power_iters, power_tol));
  return std::unique_ptr<PsfConvolve>(new PsfT<float>(op, power_iters, power_tol));
}

}  // namespace pg
