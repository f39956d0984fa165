#include "solver.h"

#include <vector>

#include "device_kernels.h"
#include "device_util.h"

namespace pg {

namespace {
template <typename real>
void run(Operator &op, const void *y, void *x, const FbParams &p, double *gammas,
         cudaStream_t s) {
  const OperatorInfo info = op.info();
  const int64_t N = int64_t(info.imsizex) * info.imsizey;
  const size_t cb = 2 * sizeof(real);
  DeviceBuffer b, nx, scratch;
  int64_t unused = 0;
  b.alloc(cb * size_t(N), &unused);
  nx.alloc(cb * size_t(N), &unused);
  // partial maxima, max, gamma, and one gamma per iteration
  scratch.alloc(sizeof(double) * (kNormBlocks + 2 + size_t(p.iterations)), &unused);
  double *partial = scratch.as<double>();
  double *mx = partial + kNormBlocks, *gamma = mx + 1, *hist = gamma + 1;
  // b = Phi^H y (the dirty image); gamma_0 = gamma_scale max |Phi^H y|
  op.adjoint(y, b.get(), s);
  cuda_check(launch_max_abs<real>(b.get(), N, false, partial, mx, s), "max");
  cuda_check(launch_gamma_update(gamma, mx, p.gamma_scale, 0.0, 0, 1, nullptr, s), "gamma");
  for (int it = 0; it < p.iterations; ++it) {
    op.normal(x, nx.get(), s);
    cuda_check(launch_fb_step<real>(x, nx.get(), b.get(), N, p.step, gamma, p.real_constraint,
                                    p.positive_constraint, s),
               "fb step");
    // record the gamma this iteration used, then the step-size update
    cuda_check(cudaMemcpyAsync(hist + it, gamma, sizeof(double), cudaMemcpyDeviceToDevice, s),
               "gamma history");
    cuda_check(launch_max_abs<real>(x, N, true, partial, mx, s), "max");
    cuda_check(launch_gamma_update(gamma, mx, p.update_scale, p.update_tol,
                                   it < p.update_iters ? 1 : 0, 0, nullptr, s),
               "gamma");
  }
  if (gammas && p.iterations > 0)
    cuda_check(cudaMemcpyAsync(gammas, hist, sizeof(double) * p.iterations,
                               cudaMemcpyDeviceToHost, s),
               "gamma history");
  cuda_check(cudaStreamSynchronize(s), "forward_backward");
}
}  // namespace

void forward_backward(Operator &op, const void *y, void *x, const FbParams &p, double *gammas,
                      cudaStream_t stream) {
  if (p.iterations < 0) throw Error(kInvalidArgument, "iterations must be >= 0");
  if (!(p.step > 0)) throw Error(kInvalidArgument, "step must be > 0");
  const OperatorInfo info = op.info();
  DeviceGuard guard(info.device);
  if (info.fp64)
    run<double>(op, y, x, p, gammas, stream);
  else
    run<float>(op, y, x, p, gammas, stream);
}

}  // namespace pg
