// Solver-side consumer of the measurement operator: a forward-backward
// (proximal gradient) loop for the l1-regularised problem
//   min_x 1/2 ||y - Phi x||^2 + gamma ||x||_1,   x real and >= 0 optionally,
// with Phi the normalised operator, driven entirely on the device through
// Operator::normal (Phi^H Phi with slot-ordered visibilities) and the
// adjoint.  Its parameters follow the reference's imaging setup: the l1
// weight starts at 1e-3 max |Phi^H y| (cpp/purify/algorithm_factory.h:73-76)
// and is updated after each iteration to step_size_scale max |Re x| when it
// moved by more than update_tol and fewer than update_iters iterations have
// run (the step-size rule of cpp/purify/update_factory.h:46-54).  The
// reference applies the operator inside sopt's proximal ADMM, which is not
// available here; this loop is the same kind of caller: many Phi^H Phi
// applies per solve with element-wise proximal steps between them.
#pragma once
#include <cuda_runtime_api.h>

#include <cstdint>

#include "operator.h"

namespace pg {

struct FbParams {
  int iterations = 20;
  double step = 1.0;            // gradient step mu (1 / ||Phi||^2 = 1 when normalised)
  double gamma_scale = 1e-3;    // gamma_0 = gamma_scale max |Phi^H y|
  double update_scale = 1e-3;   // gamma' = update_scale max |Re x|
  double update_tol = 1e-3;     // gamma <- gamma' when |gamma - gamma'| > update_tol
  int update_iters = 0;         // ... during the first update_iters iterations
  bool real_constraint = true;  // keep Re x only
  bool positive_constraint = true;  // then max(Re x, 0)
};

// x (device, imsizey * imsizex values of the operator's precision) is the
// start on entry and the solution on exit; y (device, M values) the
// visibilities.  gammas (host, may be null) receives the l1 weight used in
// each iteration.  Ordered on `stream`; returns after the device work ends.
void forward_backward(Operator &op, const void *y, void *x, const FbParams &p, double *gammas,
                      cudaStream_t stream);

// Device kernels of the loop (solver_kernels.cu).
template <typename real>
cudaError_t launch_fb_step(void *x, const void *nx, const void *b, int64_t n, double step,
                           const double *gamma, bool real_c, bool pos_c, cudaStream_t s);
// out[0] = max |Re x| (real_part) or max |x| over n values; deterministic.
template <typename real>
cudaError_t launch_max_abs(const void *x, int64_t n, bool real_part, double *partial, double *out,
                           cudaStream_t s);
// gamma <- scale * (*mx) on the first call (init), else the update rule.
cudaError_t launch_gamma_update(double *gamma, const double *mx, double scale, double tol,
                                int enabled, int init, double *history, cudaStream_t s);

}  // namespace pg
