"""The allocation-free G^H entry point (purify_gb300_grid_no_alloc).

It serves callers that may not allocate device memory once they run — codes
that give all GPU memory to a pool at start-up, or processes under a hard
memory cap on a shared GPU.  Its scratch is the library's fixed device array
instead of buffers of its own.  It must give the result of the ordinary G^H
entry point (purify_gb300_grid), on consecutive calls (the array keeps the
previous call's contents), and must refuse an operator whose scratch does
not fit.  This file sorts last so that a run stopping at its first failure
has run every other test before it.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _operator(pg, M, n, J, seed, precision="fp32"):
    rng = np.random.default_rng(seed)
    u = rng.normal(0, n / 4, M)
    v = rng.normal(0, n / 4, M)
    return pg.MeasurementOperator(u, v, None, None, n, n, 2.0, power_iters=0, kernel="kb",
                                  Ju=J, Jv=J, precision=precision)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_grid_no_alloc_matches_grid_on_consecutive_calls(pg, cuda, precision):
    torch = cuda
    op = _operator(pg, 100_000, 256, 4, 0, precision)
    assert op.grid_no_alloc_bytes() <= (32 << 20)
    dt = op.complex_dtype
    rng = np.random.default_rng(1)
    grids = 4 * 256 * 256
    for call in range(2):  # second call runs over what the first left in the array
        y = torch.from_numpy(rng.standard_normal(op.M) + 1j * rng.standard_normal(op.M)).to(dt).cuda()
        ref = torch.empty(grids, dtype=dt, device="cuda")
        out = torch.full((grids,), float("nan"), dtype=dt, device="cuda")
        op.grid_into(y, ref)
        op.grid_no_alloc_into(y, out)
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(a).all()
        assert rel_l2(a, b) <= 1e-5, (call, rel_l2(a, b))


def test_grid_no_alloc_refuses_an_operator_that_does_not_fit(pg, cuda):
    torch = cuda
    op = _operator(pg, 2_000_000, 1024, 6, 2)
    need = op.grid_no_alloc_bytes()
    assert need > (32 << 20)
    y = torch.zeros(op.M, dtype=torch.complex64, device="cuda")
    g = torch.zeros(4 * 1024 * 1024, dtype=torch.complex64, device="cuda")
    with pytest.raises(pg.PurifyError) as e:
        op.grid_no_alloc_into(y, g)
    assert e.value.status == 1 and "scratch" in str(e.value)
