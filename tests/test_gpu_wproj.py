"""GPU w-projection rows (w_term) against the CPU FP64 oracle, which builds
the reference's explicit rows (operators.cc:49-99, projection_kernels.cc:
16-85, convolution.h:28-82).  Uniform Jw is the reference's operator; the
per-row support is the w-projection workload's rule (parity against the
oracle only: the reference has no per-row support)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = {"fp32": 1e-5, "fp64": 1e-10}


def _to(torch, a, precision):
    dt = torch.complex64 if precision == "fp32" else torch.complex128
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128)).to(dt).cuda()


def _case(n, M, seed, cell=1.0):
    rng = np.random.default_rng(seed)
    N = 2 * n
    u = rng.normal(0, N / 8, M)
    v = rng.normal(0, N / 8, M)
    du = 60.0 * 60.0 * 180.0 / cell / N / np.pi
    w_max = 12.0 * du
    w = rng.uniform(-w_max, w_max, M)
    return u, v, w, w_max


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("Jw", [1, 6, 13])
def test_uniform_w_support(pg, oracle_mod, cuda, precision, Jw):
    torch = cuda
    n, M = 64, 3000
    u, v, w, _ = _case(n, M, Jw)
    rng = np.random.default_rng(99)
    wt = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    gop = pg.MeasurementOperator(u, v, w, wt, n, n, 2.0, power_iters=0, kernel="kb", Ju=4, Jv=4,
                                 w_term=True, Jw=Jw, precision=precision)
    oop = oracle_mod.Operator(u, v, w, wt, n, n, 2.0, kernel="kb", Ju=4, Jv=4, w_term=True, Jw=Jw)
    assert gop.info()["nnz"] == oop.nnz
    x = rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)
    y = gop.forward(_to(torch, x, precision)).cpu().numpy()
    assert rel_l2(y, oop.forward(x)) < TOL[precision]
    yy = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    xx = gop.adjoint(_to(torch, yy, precision)).cpu().numpy()
    assert rel_l2(xx, oop.adjoint(yy)) < TOL[precision]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_per_row_w_support(pg, oracle_mod, cuda, precision):
    from purify_gb300 import synthetic
    torch = cuda
    n, M = 128, 6000
    u, v, w, w_max = _case(n, M, 5)
    jw = synthetic.wproj_supports(w, w_max)
    assert jw.min() == 1 and jw.max() == 21  # total supports 4 .. 24
    gop = pg.MeasurementOperator(u, v, w, None, n, n, 2.0, power_iters=0, kernel="kb", Ju=4, Jv=4,
                                 w_term=True, Jw=6, precision=precision, jw_rows=jw)
    oop = oracle_mod.Operator(u, v, w, None, n, n, 2.0, kernel="kb", Ju=4, Jv=4, w_term=True,
                              jw_rows=jw)
    assert gop.info()["nnz"] == oop.nnz
    rng = np.random.default_rng(7)
    x = rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)
    yv = gop.forward(_to(torch, x, precision)).cpu().numpy()
    assert rel_l2(yv, oop.forward(x)) < TOL[precision]
    yy = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    xx = gop.adjoint(_to(torch, yy, precision)).cpu().numpy()
    assert rel_l2(xx, oop.adjoint(yy)) < TOL[precision]
    # adjoint dot-product test
    lhs = np.vdot(yy, yv)
    rhs = np.vdot(xx, x)
    tol = 1e-6 if precision == "fp32" else 1e-12
    assert abs(lhs - rhs) <= tol * np.linalg.norm(yv) * np.linalg.norm(yy)


def test_w_power_method_and_determinism(pg, oracle_mod, cuda):
    torch = cuda
    n, M = 64, 2000
    u, v, w, _ = _case(n, M, 3)
    ops = [pg.MeasurementOperator(u, v, w, None, n, n, 2.0, power_iters=0, kernel="kb", Ju=4,
                                  Jv=4, w_term=True, Jw=8, precision="fp64") for _ in range(2)]
    oop = oracle_mod.Operator(u, v, w, None, n, n, 2.0, kernel="kb", Ju=4, Jv=4, w_term=True, Jw=8)
    n_gpu = ops[0].power_method(50, 0.0)
    n_ref = oop.power_method(50, 0.0)
    assert abs(n_gpu - n_ref) / n_ref < 1e-12
    assert ops[1].power_method(50, 0.0) == n_gpu
    x = _to(torch, np.random.default_rng(1).standard_normal(n * n), "fp64")
    a = ops[0].adjoint(ops[0].forward(x))
    b = ops[1].adjoint(ops[1].forward(x))
    torch.cuda.synchronize()
    assert torch.equal(a, b)
