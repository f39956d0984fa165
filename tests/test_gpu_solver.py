"""The solver-side consumer (purify_gb300_forward_backward) against the same
forward-backward loop run in numpy over the FP64 oracle operator.

The loop: b = Phi^H y; gamma_0 = 1e-3 max |b| (cpp/purify/algorithm_factory.h:
73-76); per iteration x <- soft_{step gamma}(x - step (Phi^H Phi x - b)),
real and positivity constraints, then the step-size update of
cpp/purify/update_factory.h:46-54 (gamma' = scale max |Re x| when it moved by
more than update_tol, during the first update_iters iterations).
Tolerances: FP64 1e-10, FP32 1e-5 relative L2 after 20 iterations, as the
operator's own parity bars."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = {"fp32": 1e-5, "fp64": 1e-10}


def oracle_forward_backward(op, y, iterations, step=1.0, gamma_scale=1e-3, update_scale=1e-3,
                            update_tol=1e-3, update_iters=0, real_c=True, pos_c=True):
    b = op.adjoint(y)
    x = np.zeros_like(b)
    gamma = gamma_scale * np.abs(b).max()
    gammas = []
    for it in range(iterations):
        v = x - step * (op.adjoint(op.forward(x)) - b)
        if real_c:
            v = v.real + 0j
        mag = np.abs(v)
        thr = step * gamma
        s = np.where(mag > thr, (mag - thr) / np.where(mag > 0, mag, 1.0), 0.0)
        v = v * s
        if pos_c:
            v = np.where(v.real < 0, 0.0, v.real) + 1j * v.imag
        x = v
        gammas.append(gamma)
        g2 = update_scale * np.abs(x.real).max()
        if it < update_iters and abs(gamma - g2) > update_tol:
            gamma = g2
    return x, np.array(gammas)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("update_iters", [0, 10])
def test_forward_backward_matches_oracle_loop(pg, oracle_mod, cuda, precision, update_iters):
    torch = cuda
    from purify_gb300 import synthetic
    n, M = 64, 20000
    rng = np.random.default_rng(5)
    u, v = synthetic.mixed_uv(M, 2 * n, 2 * n, 0.7, 0.15, seed=4)
    wt = rng.uniform(0.5, 2.0, M) + 0j  # real weights 1 / sigma, as in the reference's data
    sky = synthetic.sky_image(n, n, seed=4)
    oop = oracle_mod.Operator(u, v, None, wt, n, n, 2.0, kernel="kb", Ju=4, Jv=4)
    norm = oop.power_method(50, 1e-6)
    y = oop.forward(sky) + 1e-3 * (rng.standard_normal(M) + 1j * rng.standard_normal(M))
    gop = pg.MeasurementOperator(u, v, None, wt, n, n, 2.0, power_iters=0, kernel="kb", Ju=4,
                                 Jv=4, precision=precision)
    gop.set_norm(norm)
    dt = gop.complex_dtype
    yd = torch.from_numpy(y).to(dt).cuda()
    update_tol = 0.0 if update_iters else 1e-3
    x, gammas = gop.forward_backward(yd, iterations=20, update_iters=update_iters,
                                     update_tol=update_tol, update_scale=1e-2)
    xr, gr = oracle_forward_backward(oop, y, 20, update_iters=update_iters, update_tol=update_tol,
                                     update_scale=1e-2)
    xg = x.cpu().numpy().astype(np.complex128)
    assert rel_l2(xg, xr) < TOL[precision], rel_l2(xg, xr)
    assert np.max(np.abs(gammas - gr) / gr) < TOL[precision]
    # the solution is real and non-negative, and fits the data better than zero
    assert np.all(xg.imag == 0) and np.all(xg.real >= 0)
    assert np.linalg.norm(y - oop.forward(xg)) < np.linalg.norm(y)
