"""The allocation-free G^H entry point (purify_gb300_grid_no_alloc).

It serves callers that may not allocate device memory once they run — codes
that give all GPU memory to a pool at start-up, or processes under a hard
memory cap on a shared GPU.  Its scratch is the library's fixed device array
instead of buffers of its own.  It runs the same kernels, plan and launch
shape as the ordinary G^H entry point (purify_gb300_grid), so its result must
equal that entry point's bit for bit, on consecutive calls (the array keeps
the previous call's contents); it is also checked against the FP64 oracle's
explicit G^H (operators.h:123-145), and it must refuse an operator whose
scratch does not fit.  This file sorts last so that a run stopping at its
first failure has run every other test before it.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = {"fp32": 1e-5, "fp64": 1e-10}


def _coverage(M, n, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(0, n / 4, M), rng.normal(0, n / 4, M)


def _operator(pg, M, n, J, seed, precision="fp32"):
    u, v = _coverage(M, n, seed)
    return pg.MeasurementOperator(u, v, None, None, n, n, 2.0, power_iters=0, kernel="kb",
                                  Ju=J, Jv=J, precision=precision), u, v


def _two_calls(torch, op, oracle_op, precision, seed):
    dt = op.complex_dtype
    rng = np.random.default_rng(seed)
    cells = op.info()["ftsizeu"] * op.info()["ftsizev"]
    for call in range(2):  # the second call runs over what the first left in the array
        yh = rng.standard_normal(op.M) + 1j * rng.standard_normal(op.M)
        y = torch.from_numpy(yh).to(dt).cuda()
        ref = torch.empty(cells, dtype=dt, device="cuda")
        out = torch.full((cells,), float("nan"), dtype=dt, device="cuda")
        op.grid_into(y, ref)
        op.grid_no_alloc_into(y, out)
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        assert np.array_equal(a.view(np.float64 if precision == "fp64" else np.float32),
                              b.view(np.float64 if precision == "fp64" else np.float32)), call
        assert rel_l2(a, oracle_op.G_adjoint(yh)) < TOL[precision], call


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_grid_no_alloc_matches_grid_on_consecutive_calls(pg, oracle_mod, cuda, precision):
    op, u, v = _operator(pg, 100_000, 256, 4, 0, precision)
    assert op.grid_no_alloc_bytes() <= (32 << 20)
    ref = oracle_mod.Operator(u, v, None, None, 256, 256, 2.0, kernel="kb", Ju=4, Jv=4)
    _two_calls(cuda, op, ref, precision, 1)


def test_grid_no_alloc_w_projection(pg, oracle_mod, cuda):
    # w-projection rows: the same entry point runs the row-factor G^H kernel
    n, M = 64, 4000
    u, v = _coverage(M, n, 3)
    du = 60.0 * 60.0 * 180.0 / (2 * n) / np.pi
    w = np.random.default_rng(4).uniform(-8 * du, 8 * du, M)
    op = pg.MeasurementOperator(u, v, w, None, n, n, 2.0, power_iters=0, kernel="kb", Ju=4,
                                Jv=4, w_term=True, Jw=6, precision="fp32")
    assert op.grid_no_alloc_bytes() <= (32 << 20)
    ref = oracle_mod.Operator(u, v, w, None, n, n, 2.0, kernel="kb", Ju=4, Jv=4, w_term=True,
                              Jw=6)
    _two_calls(cuda, op, ref, "fp32", 5)


def test_grid_no_alloc_refuses_an_operator_that_does_not_fit(pg, cuda):
    torch = cuda
    op, _, _ = _operator(pg, 2_000_000, 1024, 6, 2)
    need = op.grid_no_alloc_bytes()
    assert need > (32 << 20)
    y = torch.zeros(op.M, dtype=torch.complex64, device="cuda")
    g = torch.zeros(4 * 1024 * 1024, dtype=torch.complex64, device="cuda")
    with pytest.raises(pg.PurifyError) as e:
        op.grid_no_alloc_into(y, g)
    assert e.value.status == 1 and "scratch" in str(e.value)
