"""The combined degrid/grid operator Phi^H Phi (init_grid_degrid_operator_2d,
compact_operators.h:147-174) and the PSF convolution approximation
(init_psf_convolve_2d, compact_operators.h:279-307) against the FP64 oracle,
and the reference's power-method checks of both (tests/operators.cc:171-215:
the normalised operators have norm 1 within power_tol).

Tolerances (relative L2): FP64 1e-10, FP32 1e-5 (the parity bars of the
measurement operator); normal vs adjoint(forward): exact (same kernels on
the same values, only the visibility order between the halves differs);
against the column-walk G^H (tuning grid_walk = 1): 1e-6 (FP32), 1e-13
(FP64), the summation order."""
import numpy as np
import pytest

from conftest import rel_l2
from purify_gb300 import synthetic

pytestmark = pytest.mark.gpu
TOL = {"fp32": 1e-5, "fp64": 1e-10}


def case(n=64, M=6000, seed=4):
    u, v = synthetic.gaussian_core_uv(M, 2 * n, 2 * n, 0.25, seed=seed)
    return u, v, n


def dev(torch, a, precision):
    dt = torch.complex64 if precision == "fp32" else torch.complex128
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128)).to(dt).cuda()


def host(t):
    return t.cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_normal_equals_forward_then_adjoint(pg, cuda, precision):
    torch = cuda
    u, v, n = case()
    wt = np.random.default_rng(1).standard_normal(u.size) + 0.5j
    op = pg.MeasurementOperator(u, v, None, wt, n, n, 2.0, power_iters=10, precision=precision)
    x = dev(torch, synthetic.sky_image(n, n), precision)
    a = op.normal(x)
    b = op.adjoint(op.forward(x))
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    walk = pg.MeasurementOperator(u, v, None, wt, n, n, 2.0, power_iters=0, precision=precision,
                                  tuning={"grid_walk": 1})
    walk.set_norm(op.norm)
    c = walk.adjoint(walk.forward(x))
    assert rel_l2(host(c), host(a)) < (1e-6 if precision == "fp32" else 1e-13)
    # in place
    y = x.clone()
    op.normal_into(y, y)
    torch.cuda.synchronize()
    assert torch.equal(y, a)


@pytest.mark.parametrize("kernel,J", [("kb", 4), ("kb", 6), ("pswf", 6), ("gauss", 3),
                                      ("box", 1)])
def test_one_pass_normal_is_bit_identical(pg, oracle_mod, cuda, kernel, J):
    """G^H G of the normal operator in one pass over each task (tuning
    normal_pass = 1, the default below J = 6; FP32, unit weights,
    single-cell items) evaluates the
    taps once and keeps no slot-ordered vector, yet sums the same values in
    the same order as degrid then grid (normal_pass = 2) with the same
    two-warp CTAs: normal, in place and out of place, and the power method
    are bit-identical to that path, and match
    the oracle.  A dense cell puts several visibilities on one item."""
    torch = cuda
    u, v, n = case(n=96, M=9000, seed=J)
    u[:300], v[:300] = 1.3, -2.6
    ops = [pg.MeasurementOperator(u, v, None, None, n, n, 2.0, power_iters=0, precision="fp32",
                                  kernel=kernel, Ju=J, Jv=J,
                                  tuning={"normal_pass": p, "threads": 64})
           for p in (2, 1)]
    x = dev(torch, synthetic.sky_image(n, n, seed=J), "fp32")
    a, b = ops[0].normal(x), ops[1].normal(x)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    y = x.clone()
    ops[1].normal_into(y, y)
    torch.cuda.synchronize()
    assert torch.equal(y, b)
    assert ops[0].power_method(8, 0.0) == ops[1].power_method(8, 0.0)
    oop = oracle_mod.Operator(u, v, None, None, n, n, 2.0, kernel=kernel, Ju=J, Jv=J)
    oop.set_norm(ops[1].norm)
    c = host(ops[1].normal(x))
    assert rel_l2(c, oop.adjoint(oop.forward(host(x)))) < TOL["fp32"]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_normal_vs_oracle_and_norm(pg, oracle_mod, cuda, precision):
    torch = cuda
    u, v, n = case()
    op = pg.MeasurementOperator(u, v, None, None, n, n, 2.0, power_iters=100, power_tol=1e-4,
                                precision=precision)
    oop = oracle_mod.Operator(u, v, None, None, n, n, 2.0, kernel="kb", Ju=4, Jv=4)
    oop.power_method(100, 1e-4)
    x = synthetic.sky_image(n, n, seed=2)
    got = host(op.normal(dev(torch, x, precision)))
    assert rel_l2(got, oop.adjoint(oop.forward(x))) < TOL[precision]
    # the normalised Phi^H Phi has norm 1 (tests/operators.cc:184-190)
    z = torch.ones(n * n, dtype=op.complex_dtype, device="cuda") / n
    old = 0.0
    for _ in range(100):
        z = op.normal(z)
        value = float(torch.linalg.norm(z).item())
        z = z / value
        if abs(old - value) / value < 1e-8:
            break
        old = value
    assert abs(np.sqrt(value) - 1.0) < 1e-3


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_psf_convolve_vs_oracle(pg, oracle_mod, cuda, precision):
    torch = cuda
    u, v, n = case(n=64, M=5000, seed=7)
    op = pg.MeasurementOperator(u, v, None, None, n, n, 2.0, power_iters=100, power_tol=1e-4,
                                precision=precision)
    oop = oracle_mod.Operator(u, v, None, None, n, n, 2.0, kernel="kb", Ju=4, Jv=4)
    oop.power_method(100, 1e-4)
    psf = pg.PsfConvolve(op, power_iters=100, power_tol=1e-4)
    apply_ref, norm_ref = oracle_mod.psf_convolve(oop, n, n, 100, 1e-4)
    assert abs(psf.norm - norm_ref) / norm_ref < (1e-10 if precision == "fp64" else 1e-5)
    x = synthetic.sky_image(n, n, seed=3)
    got = host(psf(dev(torch, x, precision)))
    assert rel_l2(got, apply_ref(x)) < TOL[precision]
    # the normalised convolution has norm 1 (tests/operators.cc:201-214); a
    # random start (the all-ones image is the zero-frequency eigenvector)
    g = np.random.default_rng(0)
    z = dev(torch, g.standard_normal(n * n) + 1j * g.standard_normal(n * n), precision)
    z = z / torch.linalg.norm(z)
    for _ in range(200):
        z = psf(z)
        value = float(torch.linalg.norm(z).item())
        z = z / value
    assert abs(np.sqrt(value) - 1.0) < 1e-3


def test_psf_of_non_square_image(pg, oracle_mod, cuda):
    torch = cuda
    ny, nx = 48, 80
    u, v = synthetic.gaussian_core_uv(3000, 2 * nx, 2 * ny, 0.25, seed=9)
    op = pg.MeasurementOperator(u, v, None, None, ny, nx, 2.0, power_iters=50, precision="fp64")
    oop = oracle_mod.Operator(u, v, None, None, ny, nx, 2.0, kernel="kb", Ju=4, Jv=4)
    oop.power_method(50, 1e-4)
    psf = pg.PsfConvolve(op, power_iters=50)
    apply_ref, norm_ref = oracle_mod.psf_convolve(oop, ny, nx, 50, 1e-4)
    x = synthetic.sky_image(ny, nx, seed=5)
    assert rel_l2(host(psf(dev(torch, x, "fp64"))), apply_ref(x)) < 1e-10
