"""Full-size (1024^2 image, 2048^2 grid, 10^7 visibilities, KB J=6) checks
through size-independent properties: FP32 vs FP64 GPU paths, the adjoint
dot-product test, linearity, FP32/FP64 rows against the CPU FP64 oracle
(forward rows are independent, so a row sample of the oracle is exact) and
the adjoint of a row-sampled y against the oracle (G^H is linear, so that
check is exact too)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def large(pg, cuda):
    from purify_gb300 import synthetic
    torch = cuda
    c = synthetic.config_large(M=10_000_000, seed=0)
    kw = dict(imsizey=1024, imsizex=1024, kernel="kb", Ju=6, Jv=6, power_iters=0)
    op32 = pg.MeasurementOperator(c["u"], c["v"], None, None, precision="fp32", **kw)
    op64 = pg.MeasurementOperator(c["u"], c["v"], None, None, precision="fp64", **kw)
    norm = op32.power_method(10, 1e-4)
    op64.set_norm(norm)
    return c, op32, op64, torch


def test_fp32_matches_fp64_at_full_size(large):
    c, op32, op64, torch = large
    x = torch.from_numpy(c["x"]).cuda()
    y32 = op32.forward(x.to(torch.complex64)).cpu().numpy()
    y64 = op64.forward(x).cpu().numpy()
    assert rel_l2(y32, y64) < 1e-5
    yin = torch.from_numpy(y64).cuda()
    x32 = op32.adjoint(yin.to(torch.complex64)).cpu().numpy()
    x64 = op64.adjoint(yin).cpu().numpy()
    assert rel_l2(x32, x64) < 1e-5


def test_adjoint_dot_product_full_size(large):
    c, op32, op64, torch = large
    rng = np.random.default_rng(3)
    M = c["u"].size
    for op, tol, dt in ((op32, 1e-6, torch.complex64), (op64, 1e-12, torch.complex128)):
        x = torch.from_numpy(rng.standard_normal(1024 * 1024) + 1j * rng.standard_normal(1024 * 1024)).to(dt).cuda()
        y = torch.from_numpy(rng.standard_normal(M) + 1j * rng.standard_normal(M)).to(dt).cuda()
        px = op.forward(x)
        phy = op.adjoint(y)
        lhs = torch.vdot(y.to(torch.complex128), px.to(torch.complex128)).item()
        rhs = torch.vdot(phy.to(torch.complex128), x.to(torch.complex128)).item()
        scale = float(torch.linalg.vector_norm(px.to(torch.complex128))) * float(
            torch.linalg.vector_norm(y.to(torch.complex128)))
        assert abs(lhs - rhs) <= tol * scale


def test_linearity_full_size(large):
    c, op32, op64, torch = large
    rng = np.random.default_rng(4)
    a = torch.from_numpy(rng.standard_normal(1024 * 1024) + 0j).to(torch.complex128).cuda()
    b = torch.from_numpy(c["x"]).cuda()
    lhs = op64.forward(2.0 * a - 3.0j * b)
    rhs = 2.0 * op64.forward(a) - 3.0j * op64.forward(b)
    assert rel_l2(lhs.cpu().numpy(), rhs.cpu().numpy()) < 1e-12


def test_rows_against_oracle(large, oracle_mod):
    c, op32, op64, torch = large
    idx = np.random.default_rng(5).choice(c["u"].size, 20000, replace=False)
    ref = oracle_mod.Operator(c["u"][idx], c["v"][idx], None, None, 1024, 1024, 2.0,
                              kernel="kb", Ju=6, Jv=6)
    ref.set_norm(op32.norm)
    yr = ref.forward(c["x"])
    x = torch.from_numpy(c["x"]).cuda()
    y32 = op32.forward(x.to(torch.complex64)).cpu().numpy()[idx]
    y64 = op64.forward(x).cpu().numpy()[idx]
    assert rel_l2(y32, yr) < 1e-5
    assert rel_l2(y64, yr) < 1e-10


def test_adjoint_sample_against_oracle(large, oracle_mod):
    """G^H is linear, so a y that is zero outside a row sample gives an exact
    oracle check of the full-size adjoint (tiling, fold halos and the task
    order all act on it): the oracle operator built on the sample rows alone,
    with the same norm, must give the same image.  Generalises the G^H golden
    of the reference (cpp/tests/operators.cc:80-91) to the full workload."""
    c, op32, op64, torch = large
    M = c["u"].size
    idx = np.random.default_rng(6).choice(M, 20000, replace=False)
    rng = np.random.default_rng(7)
    ys = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    ref = oracle_mod.Operator(c["u"][idx], c["v"][idx], None, None, 1024, 1024, 2.0,
                              kernel="kb", Ju=6, Jv=6)
    ref.set_norm(op32.norm)
    xr = ref.adjoint(ys)
    y = np.zeros(M, dtype=np.complex128)
    y[idx] = ys
    yd = torch.from_numpy(y).cuda()
    x32 = op32.adjoint(yd.to(torch.complex64)).cpu().numpy()
    x64 = op64.adjoint(yd).cpu().numpy()
    assert rel_l2(x32, xr) < 1e-5
    assert rel_l2(x64, xr) < 1e-10
