"""GPU measurement operator against the CPU FP64 oracle and the reference's
golden vectors.  Every call goes through the C ABI (libpurify_gb300.so).

Tolerances (relative L2 unless stated):
  FP64 GPU path vs oracle        1e-10
  FP32 GPU path vs oracle        1e-5   (the stated FP32 tolerance of the path)
  golden G / G^H (operators.cc)  1e-5   isApprox, as the reference test
  golden M31 Phi x               1e-6   isApprox after max-normalisation
  adjoint dot-product test       1e-6 (FP32), 1e-12 (FP64), relative to ||Phi x|| ||y||
"""
import numpy as np
import pytest

from conftest import golden, is_approx, rel_l2

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-5, "fp64": 1e-10}
DOT_TOL = {"fp32": 1e-6, "fp64": 1e-12}


def to_dev(torch, a, precision):
    dt = torch.complex64 if precision == "fp32" else torch.complex128
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128)).to(dtype=dt).cuda()


def to_np(t):
    return t.cpu().numpy().astype(np.complex128)


def make_pair(pg, oracle_mod, u, v, n_y, n_x, kernel="kb", J=4, weights=None,
              precision="fp32", oversample=2.0):
    gop = pg.MeasurementOperator(u, v, None, weights, n_y, n_x, oversample, power_iters=0,
                                 kernel=kernel, Ju=J, Jv=J, precision=precision)
    oop = oracle_mod.Operator(u, v, None, weights, n_y, n_x, oversample, kernel=kernel, Ju=J, Jv=J)
    return gop, oop


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_golden_gridding_matrix(pg, cuda, precision):
    g = golden("operators")
    op = pg.MeasurementOperator(g["u"], g["v"], None, None, 16, 16, 2.0, power_iters=0,
                                kernel="kb", Ju=4, Jv=4, precision=precision)
    torch = cuda
    vis = torch.empty(10, dtype=op.complex_dtype, device="cuda")
    op.degrid_into(to_dev(torch, g["direct_input"], precision), vis)
    torch.cuda.synchronize()
    assert is_approx(to_np(vis), g["expected_direct"], 1e-5)
    grid = torch.empty(1024, dtype=op.complex_dtype, device="cuda")
    op.grid_into(to_dev(torch, g["indirect_input"], precision), grid)
    torch.cuda.synchronize()
    assert is_approx(to_np(grid), g["expected_indirect"], 1e-5)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("name,J", [("kb", 4), ("pswf", 6), ("gauss", 6)])
def test_golden_m31(pg, cuda, precision, name, J):
    m = golden("measurement_operator")
    x = m["m31"].astype(np.complex128)
    op = pg.MeasurementOperator(m["v"], m["u"], None, None, 256, 256, 2.0, power_iters=1,
                                power_tol=1e-9, kernel=name, Ju=J, Jv=J, precision=precision)
    y = op.forward(x)  # host complex<double> entry point
    e = m[name + "_exact"]
    assert is_approx(y / np.abs(y).max(), e / np.abs(e).max(), 1e-6)


@pytest.fixture(scope="module")
def small_config():
    from purify_gb300 import synthetic
    return synthetic.config_small(seed=0)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_small_config_parity(pg, oracle_mod, cuda, small_config, precision):
    """256^2 image, 512^2 grid, 1e5 visibilities, KB J=4 (the CPU-runnable case)."""
    c = small_config
    torch = cuda
    rng = np.random.default_rng(1)
    wt = np.exp(1j * rng.uniform(0, 2 * np.pi, c["u"].size)) * rng.uniform(0.5, 2, c["u"].size)
    gop, oop = make_pair(pg, oracle_mod, c["u"], c["v"], 256, 256, "kb", 4, wt, precision)
    y_ref = oop.forward(c["x"])
    y = to_np(gop.forward(to_dev(torch, c["x"], precision)))
    assert rel_l2(y, y_ref) < TOL[precision], rel_l2(y, y_ref)
    yy = (rng.standard_normal(c["u"].size) + 1j * rng.standard_normal(c["u"].size))
    x_ref = oop.adjoint(yy)
    x = to_np(gop.adjoint(to_dev(torch, yy, precision)))
    assert rel_l2(x, x_ref) < TOL[precision], rel_l2(x, x_ref)
    # adjoint dot-product test <Phi x, y> = <x, Phi^H y>
    lhs = np.vdot(yy, y)
    rhs = np.vdot(x, c["x"])
    assert abs(lhs - rhs) <= DOT_TOL[precision] * np.linalg.norm(y) * np.linalg.norm(yy)


@pytest.mark.parametrize("kernel,J", [("kb", 1), ("kb", 2), ("kb", 3), ("kb", 5), ("kb", 6),
                                      ("kb", 7), ("kb", 8), ("pswf", 6), ("gauss", 4),
                                      ("gauss", 2), ("box", 3), ("kbmin", 4),
                                      ("gauss_alt", 5)])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_kernels_and_supports(pg, oracle_mod, cuda, kernel, J, precision):
    torch = cuda
    rng = np.random.default_rng(J)
    M, n = 4000, 48
    u = rng.normal(0, 20, M)
    v = rng.normal(0, 20, M)
    gop, oop = make_pair(pg, oracle_mod, u, v, n, n, kernel, J, None, precision)
    x = rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)
    y = to_np(gop.forward(to_dev(torch, x, precision)))
    assert rel_l2(y, oop.forward(x)) < TOL[precision]
    yy = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    xx = to_np(gop.adjoint(to_dev(torch, yy, precision)))
    assert rel_l2(xx, oop.adjoint(yy)) < TOL[precision]


@pytest.mark.parametrize("ny,nx,os", [
    (32, 32, 2.0),       # 64^2 grid, the smallest fused size
    (64, 128, 2.0),      # 128 x 256, non-square
    (80, 40, 1.6),       # 128 x 64 grid around a non-power-of-two image (x0 = 12, y0 = 24)
    (256, 256, 2.0),     # 512^2
    (1024, 2048, 2.0),   # 2048 x 4096: the largest row length, the column pass's largest height
    (2048, 1024, 2.0),   # 4096 x 2048: columns of 4096 through cuFFT's column plan
])
def test_fused_fft_grids(pg, oracle_mod, cuda, ny, nx, os):
    """FP32 operators on grids of power-of-two width run the fused row passes
    (correction + padding + row FFT, row FFT + cropping + correction) with a
    column transform (the column pass up to 2048 rows, cuFFT above) instead of
    pad + 2-D FFT + crop; both directions against the oracle and the adjoint
    dot-product test."""
    torch = cuda
    rng = np.random.default_rng(ny + nx)
    M = 5000
    Nu, Nv = int(np.floor(os * nx)), int(np.floor(os * ny))
    u = rng.uniform(-Nu / 2, Nu / 2, M)
    v = rng.uniform(-Nv / 2, Nv / 2, M)
    gop, oop = make_pair(pg, oracle_mod, u, v, ny, nx, "kb", 4, None, "fp32", os)
    x = rng.standard_normal(ny * nx) + 1j * rng.standard_normal(ny * nx)
    y = to_np(gop.forward(to_dev(torch, x, "fp32")))
    assert rel_l2(y, oop.forward(x)) < TOL["fp32"]
    yy = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    xx = to_np(gop.adjoint(to_dev(torch, yy, "fp32")))
    assert rel_l2(xx, oop.adjoint(yy)) < TOL["fp32"]
    lhs = np.vdot(yy, y)
    rhs = np.vdot(xx, x)
    assert abs(lhs - rhs) <= DOT_TOL["fp32"] * np.linalg.norm(y) * np.linalg.norm(yy)


@pytest.mark.parametrize("ny,nx", [(256, 256), (80, 40), (512, 1024)])
def test_column_pass_matches_cufft_columns(pg, cuda, ny, nx):
    """The column pass (only the image rows read in the forward, written in
    the adjoint) against cuFFT's strided column plan on the same operator
    (tuning fft_columns = 1): the same transform up to FP32 rounding."""
    torch = cuda
    rng = np.random.default_rng(ny * 7 + nx)
    M = 6000
    u = rng.normal(0, nx / 3, M)
    v = rng.normal(0, ny / 3, M)
    ops = [pg.MeasurementOperator(u, v, None, None, ny, nx, 2.0 if ny != 80 else 1.6,
                                  power_iters=0, kernel="kb", Ju=6, Jv=6, precision="fp32",
                                  tuning={"fft_columns": c}) for c in (0, 1)]
    x = to_dev(torch, rng.standard_normal(ny * nx) + 1j * rng.standard_normal(ny * nx), "fp32")
    y = to_dev(torch, rng.standard_normal(M) + 1j * rng.standard_normal(M), "fp32")
    f = [to_np(op.forward(x)) for op in ops]
    a = [to_np(op.adjoint(y)) for op in ops]
    assert rel_l2(f[0], f[1]) < 1e-6
    assert rel_l2(a[0], a[1]) < 1e-6


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("ny,nx,os,spread", [
    (20, 36, 2.0, 30.0),     # non-square, non power of two grid (40 x 72)
    (33, 17, 2.0, 200.0),    # odd sizes, coordinates far outside the grid (periodic wrap)
    (64, 64, 1.5, 20.0),     # oversampling 1.5 (grid 96^2)
])
def test_shapes_and_wrap(pg, oracle_mod, cuda, precision, ny, nx, os, spread):
    torch = cuda
    rng = np.random.default_rng(ny * nx)
    M = 3000
    u = rng.normal(0, spread, M)
    v = rng.normal(0, spread, M)
    gop, oop = make_pair(pg, oracle_mod, u, v, ny, nx, "kb", 4, None, precision, os)
    x = rng.standard_normal(ny * nx) + 1j * rng.standard_normal(ny * nx)
    y = to_np(gop.forward(to_dev(torch, x, precision)))
    assert rel_l2(y, oop.forward(x)) < TOL[precision]
    yy = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    xx = to_np(gop.adjoint(to_dev(torch, yy, precision)))
    assert rel_l2(xx, oop.adjoint(yy)) < TOL[precision]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_dense_single_cell_and_single_visibility(pg, oracle_mod, cuda, precision):
    torch = cuda
    rng = np.random.default_rng(5)
    for M, spread in ((5000, 0.0), (1, 3.0)):
        u = 0.3 + spread * rng.standard_normal(M)
        v = -0.7 + spread * rng.standard_normal(M)
        gop, oop = make_pair(pg, oracle_mod, u, v, 32, 32, "kb", 6, None, precision)
        x = rng.standard_normal(1024) + 1j * rng.standard_normal(1024)
        y = to_np(gop.forward(to_dev(torch, x, precision)))
        assert rel_l2(y, oop.forward(x)) < TOL[precision]
        yy = rng.standard_normal(M) + 1j * rng.standard_normal(M)
        xx = to_np(gop.adjoint(to_dev(torch, yy, precision)))
        assert rel_l2(xx, oop.adjoint(yy)) < TOL[precision]


def test_empty_coverage(pg, cuda):
    torch = cuda
    op = pg.MeasurementOperator(np.zeros(0), np.zeros(0), None, None, 16, 16, power_iters=0)
    x = torch.ones(256, dtype=torch.complex64, device="cuda")
    assert op.forward(x).numel() == 0
    xa = op.adjoint(torch.zeros(0, dtype=torch.complex64, device="cuda"))
    torch.cuda.synchronize()
    assert float(xa.abs().max()) == 0.0
    with pytest.raises(pg.PurifyError) as e:
        op.power_method(10, 1e-4)
    assert e.value.status == 5  # operators.h:187, "Operator norm is not greater than zero."


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_power_method_matches_oracle(pg, oracle_mod, cuda, small_config, precision):
    c = small_config
    gop, oop = make_pair(pg, oracle_mod, c["u"][:20000], c["v"][:20000], 256, 256, "kb", 4, None,
                         precision)
    # a fixed number of rounds (tol 0 never stops early): the two estimates
    # then differ only by arithmetic precision
    n_gpu = gop.power_method(100, 0.0)
    n_ref = oop.power_method(100, 0.0)
    assert abs(n_gpu - n_ref) / n_ref < (1e-5 if precision == "fp32" else 1e-12)
    if precision == "fp64":  # and the same stopping round with the reference's rule
        assert abs(gop.power_method(100, 1e-4) - oop.power_method(100, 1e-4)) / n_ref < 1e-12
    # the normalised operator has ||Phi^H Phi|| = 1 (operators.cc:147-154): a
    # power iteration on it from a random start, stopped when the eigenvalue
    # changes by less than tol^2, returns 1 within tol
    torch = cuda
    tol = 1e-4
    gop.power_method(3000, 1e-6)
    x = to_dev(torch, np.random.default_rng(0).standard_normal(65536), precision)
    x = x / torch.linalg.vector_norm(x)
    old = 0.0
    for _ in range(2000):
        x = gop.adjoint(gop.forward(x))
        lam = float(torch.linalg.vector_norm(x))
        x = x / lam
        if old and abs(old - lam) / old < tol * tol:
            break
        old = lam
    assert abs(np.sqrt(lam) - 1.0) < 10 * tol


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_determinism(pg, cuda, small_config, precision):
    """Two applies, and two independently built operators, agree bit for bit
    (the reference checks 1e-12 after 100 Phi^H Phi rounds, operators.cc:155-168)."""
    torch = cuda
    c = small_config
    ops = [pg.MeasurementOperator(c["u"], c["v"], None, None, 256, 256, power_iters=5,
                                  precision=precision) for _ in range(2)]
    assert ops[0].norm == ops[1].norm
    x0 = to_dev(torch, c["x"], precision)
    a, b = x0.clone(), x0.clone()
    for _ in range(20):
        a = ops[0].adjoint(ops[0].forward(a))
        b = ops[1].adjoint(ops[1].forward(b))
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    y1 = ops[0].forward(x0)
    y2 = ops[0].forward(x0)
    torch.cuda.synchronize()
    assert torch.equal(y1, y2)


def test_host_entry_points_match_device(pg, cuda, small_config):
    torch = cuda
    c = small_config
    op = pg.MeasurementOperator(c["u"], c["v"], None, None, 256, 256, power_iters=3)
    y_host = op.forward(c["x"])
    y_dev = to_np(op.forward(to_dev(torch, c["x"], "fp32")))
    assert np.array_equal(y_host, y_dev)
    x_host = op.adjoint(y_host)
    x_dev = to_np(op.adjoint(to_dev(torch, y_host, "fp32")))
    assert np.array_equal(x_host, x_dev)


def test_caller_stream_ordering(pg, cuda, small_config):
    """Applies on a side stream are ordered after prior work on that stream."""
    torch = cuda
    c = small_config
    op = pg.MeasurementOperator(c["u"], c["v"], None, None, 256, 256, power_iters=0)
    s = torch.cuda.Stream()
    x = to_dev(torch, c["x"], "fp32")
    ref = to_np(op.forward(x))
    with torch.cuda.stream(s):
        x2 = x * 2  # enqueued on s
        y2 = torch.empty(op.M, dtype=torch.complex64, device="cuda")
        op.forward_into(x2, y2, stream=s)
    s.synchronize()
    assert rel_l2(to_np(y2), 2 * ref) < 1e-6


def test_operators_with_different_kernels_interleaved(pg, oracle_mod, cuda):
    """Operators with different kernels, applied alternately on two streams,
    each give their own result."""
    torch = cuda
    rng = np.random.default_rng(21)
    M, n = 6000, 64
    u = rng.normal(0, 25, M)
    v = rng.normal(0, 25, M)
    specs = [("kb", 4), ("gauss", 6), ("kbmin", 5)]
    ops = [pg.MeasurementOperator(u, v, None, None, n, n, power_iters=0, kernel=k, Ju=J, Jv=J)
           for k, J in specs]
    refs = [oracle_mod.Operator(u, v, None, None, n, n, kernel=k, Ju=J, Jv=J) for k, J in specs]
    x = rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)
    xd = to_dev(torch, x, "fp32")
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    outs = []
    for rep in range(3):
        for k, op in enumerate(ops):
            s = streams[(rep + k) % 2]
            y = torch.empty(M, dtype=torch.complex64, device="cuda")
            xd.record_stream(s)
            with torch.cuda.stream(s):
                op.forward_into(xd, y, stream=s)
            outs.append((k, y, s))
    torch.cuda.synchronize()
    for k, y, _ in outs:
        assert rel_l2(to_np(y), refs[k].forward(x)) < 1e-5


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_recorded_applies(pg, cuda, precision):
    """Repeated applies on the same buffers are recorded into a CUDA graph and
    replayed: the results stay bit-identical to the first (direct) apply, and
    a later set_norm is honoured by the replays."""
    torch = cuda
    from purify_gb300 import synthetic
    c = synthetic.config_small()
    op = pg.MeasurementOperator(c["u"][:20000], c["v"][:20000], None, None, 256, 256, 2.0,
                                power_iters=0, precision=precision)
    x = to_dev(torch, c["x"], precision)
    y = torch.empty(20000, dtype=op.complex_dtype, device="cuda")
    xo = torch.empty_like(x)
    nz = torch.empty_like(x)
    first_y = first_x = first_n = None
    for k in range(5):
        op.forward_into(x, y)
        op.adjoint_into(y, xo)
        op.normal_into(x, nz)
        torch.cuda.synchronize()
        if k == 0:
            first_y, first_x, first_n = y.clone(), xo.clone(), nz.clone()
        else:
            assert torch.equal(y, first_y) and torch.equal(xo, first_x) and torch.equal(nz, first_n)
    op.set_norm(2.0)
    for _ in range(3):
        op.forward_into(x, y)
        op.normal_into(x, nz)
    torch.cuda.synchronize()
    assert rel_l2(to_np(y), to_np(first_y) / 2.0) < 1e-6
    assert rel_l2(to_np(nz), to_np(first_n) / 4.0) < 1e-6


@pytest.mark.parametrize("kernel,J", [("kb", 1), ("kb", 2), ("kb", 4), ("kb", 6), ("pswf", 6),
                                      ("gauss", 3), ("box", 5)])
@pytest.mark.parametrize("group", [1, 2, 3])
def test_work_item_shapes(pg, oracle_mod, cuda, kernel, J, group):
    """FP32 work items of single base cells (group 1), of aligned 2 x 2 cell
    groups sharing a (J + 1)^2 register block (group 2) and of aligned pairs
    of cells of a row sharing a J x (J + 1) block (group 3): against the
    oracle, with complex weights, a dense core and a sparse tail, wrap-
    around, and bit-identical repeats; the plan reports the shape it used."""
    torch = cuda
    rng = np.random.default_rng(10 * J + group)
    M, n = 6000, 50  # 100 x 100 grid: tiles of 25 cells, odd groups at tile edges
    u = np.concatenate([rng.normal(0, 6, M // 2), rng.uniform(-70, 70, M - M // 2)])
    v = np.concatenate([rng.normal(0, 6, M // 2), rng.uniform(-70, 70, M - M // 2)])
    wt = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    gop = pg.MeasurementOperator(u, v, None, wt, n, n, 2.0, power_iters=0, kernel=kernel, Ju=J,
                                 Jv=J, precision="fp32", tuning={"cell_group": group})
    assert gop.info()["cell_group"] == group
    oop = oracle_mod.Operator(u, v, None, wt, n, n, 2.0, kernel=kernel, Ju=J, Jv=J)
    x = rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)
    xd = to_dev(torch, x, "fp32")
    y1 = gop.forward(xd)
    y2 = gop.forward(xd)
    assert torch.equal(y1, y2)
    assert rel_l2(to_np(y1), oop.forward(x)) < TOL["fp32"]
    yy = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    yd = to_dev(torch, yy, "fp32")
    a1 = gop.adjoint(yd)
    a2 = gop.adjoint(yd)
    assert torch.equal(a1, a2)
    assert rel_l2(to_np(a1), oop.adjoint(yy)) < TOL["fp32"]


def test_work_item_shape_requests(pg, cuda):
    """Single base cells by default; 2 x 2 groups on request for complex<float>
    with J <= 6, refused (UNSUPPORTED) for complex<double> and J > 6."""
    u = np.zeros(10)
    for prec, J in (("fp32", 6), ("fp32", 8), ("fp64", 4)):
        op = pg.MeasurementOperator(u, u, None, None, 32, 32, 2.0, power_iters=0, kernel="kb",
                                    Ju=J, Jv=J, precision=prec)
        assert op.info()["cell_group"] == 1
    op = pg.MeasurementOperator(u, u, None, None, 32, 32, 2.0, power_iters=0, kernel="kb", Ju=6,
                                Jv=6, precision="fp32", tuning={"cell_group": 2})
    assert op.info()["cell_group"] == 2
    for prec, J in (("fp32", 7), ("fp64", 4)):
        with pytest.raises(pg.PurifyError) as e:
            pg.MeasurementOperator(u, u, None, None, 32, 32, 2.0, power_iters=0, kernel="kb",
                                   Ju=J, Jv=J, precision=prec, tuning={"cell_group": 2})
        assert e.value.status == 2


@pytest.mark.parametrize("kernel,J", [("kb", 1), ("kb", 2), ("gauss", 2), ("pswf", 6)])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_weights_with_sub_segmented_taps(pg, oracle_mod, cuda, kernel, J, precision):
    """Kernels whose tap fit has sub-segments (narrow supports, the PSWF)
    run without a weight stream; their operators apply complex weights in
    element-wise passes (caller order after G, slot order before G^H).
    Every path is checked against the oracle: forward and adjoint through
    caller order, the normal operator and the power method through slot
    order, and the allocation-free G^H against the ordinary one."""
    torch = cuda
    rng = np.random.default_rng(J + (0 if precision == "fp32" else 100))
    M, n = 5000, 40
    u = rng.normal(0, 15, M)
    v = rng.normal(0, 15, M)
    wt = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    gop, oop = make_pair(pg, oracle_mod, u, v, n, n, kernel, J, wt, precision)
    x = rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)
    y = to_np(gop.forward(to_dev(torch, x, precision)))
    assert rel_l2(y, oop.forward(x)) < TOL[precision]
    yy = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    xx = to_np(gop.adjoint(to_dev(torch, yy, precision)))
    assert rel_l2(xx, oop.adjoint(yy)) < TOL[precision]
    nx = to_np(gop.normal(to_dev(torch, x, precision)))
    assert rel_l2(nx, oop.adjoint(oop.forward(x))) < TOL[precision]
    n_gpu, n_ref = gop.power_method(20, 0.0), oop.power_method(20, 0.0)
    assert abs(n_gpu - n_ref) / n_ref < TOL[precision]
    cells = 4 * n * n
    yd = to_dev(torch, yy, precision)
    g1 = torch.empty(cells, dtype=gop.complex_dtype, device="cuda")
    g2 = torch.empty(cells, dtype=gop.complex_dtype, device="cuda")
    gop.grid_into(yd, g1)
    gop.grid_no_alloc_into(yd, g2)
    torch.cuda.synchronize()
    assert torch.equal(g1, g2)
    assert rel_l2(to_np(g1), oop.G_adjoint(yy)) < TOL[precision]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_caller_order_grid_is_bit_identical(pg, cuda, small_config, precision):
    """G^H reading the caller-ordered visibilities directly (the grid kernel
    gathers them, fused_permute = 1) sums the same values in the same order
    as the gather into slot order followed by the slot-ordered grid kernel
    (work items): the two adjoints are bit-identical, as are the forwards."""
    torch = cuda
    c = small_config
    ops = [pg.MeasurementOperator(c["u"], c["v"], None, None, 256, 256, 2.0, power_iters=0,
                                  kernel="kb", Ju=4, Jv=4, precision=precision,
                                  tuning={"fused_permute": fp}) for fp in (0, 1)]
    rng = np.random.default_rng(2)
    y = to_dev(torch, rng.standard_normal(c["u"].size) + 1j * rng.standard_normal(c["u"].size),
               precision)
    x = to_dev(torch, c["x"], precision)
    a0, a1 = ops[0].adjoint(y), ops[1].adjoint(y)
    f0, f1 = ops[0].forward(x), ops[1].forward(x)
    torch.cuda.synchronize()
    assert torch.equal(a0, a1) and torch.equal(f0, f1)


@pytest.mark.parametrize("kernel,Ju,Jv", [("gauss", 4, 6), ("gauss", 6, 3), ("box", 3, 5),
                                          ("gauss_alt", 2, 4), ("kb", 10, 10), ("gauss", 12, 12),
                                          ("box", 16, 16), ("kbmin", 9, 9)])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_unequal_and_wide_supports(pg, oracle_mod, cuda, kernel, Ju, Jv, precision):
    """Ju != Jv and supports above 8 taps run as plain separable rows on the
    row-factor kernels.  The reference builds G with the Jv kernel on the u
    axis and the Ju kernel on the v axis (operators.h:322-324), which the
    oracle restates; S uses ftu of Ju along x and ftv of Jv along y.  Forward,
    adjoint (complex weights) and the power method against the oracle."""
    torch = cuda
    rng = np.random.default_rng(Ju * 10 + Jv)
    M, n = 4000, 48
    u = rng.normal(0, 15, M)
    v = rng.normal(0, 15, M)
    wt = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    gop = pg.MeasurementOperator(u, v, None, wt, n, n, 2.0, power_iters=0, kernel=kernel, Ju=Ju,
                                 Jv=Jv, precision=precision)
    oop = oracle_mod.Operator(u, v, None, wt, n, n, 2.0, kernel=kernel, Ju=Ju, Jv=Jv)
    assert gop.info()["nnz"] == oop.nnz == M * Ju * Jv
    x = rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)
    y = to_np(gop.forward(to_dev(torch, x, precision)))
    assert rel_l2(y, oop.forward(x)) < TOL[precision]
    yy = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    xx = to_np(gop.adjoint(to_dev(torch, yy, precision)))
    assert rel_l2(xx, oop.adjoint(yy)) < TOL[precision]
    n_gpu, n_ref = gop.power_method(20, 0.0), oop.power_method(20, 0.0)
    assert abs(n_gpu - n_ref) / n_ref < TOL[precision]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("J,kernel,weighted", [(6, "kb", False), (4, "kb", True), (1, "kb", False),
                                              (6, "pswf", False), (5, "kbmin", False),
                                              (8, "gauss", True)])
def test_column_walk_adjoint(pg, oracle_mod, cuda, precision, J, kernel, weighted):
    """With tuning grid_walk = 1, Phi^H runs G^H as the column walk (tiles
    of 32, lanes = rows, one column flushed per step): against the oracle,
    against the work-item kernel on the same coverage (only the summation
    order differs), and repeatable bit for bit."""
    torch = cuda
    if precision == "fp64" and J > 6:
        pytest.skip("FP64 walks up to J = 6")
    rng = np.random.default_rng(J + 10 * weighted)
    M, n = 30000, 96
    u = np.concatenate([rng.normal(0, 8, M // 2), rng.uniform(-n, n, M - M // 2)])
    v = np.concatenate([rng.normal(0, 8, M // 2), rng.uniform(-n, n, M - M // 2)])
    u[:300], v[:300] = u[300:600], v[300:600]  # cells with several visibilities
    wt = (rng.uniform(0.5, 2, M) * np.exp(1j * rng.uniform(0, 2 * np.pi, M))) if weighted else None
    ops = [pg.MeasurementOperator(u, v, None, wt, n, n, 2.0, power_iters=0, kernel=kernel, Ju=J,
                                  Jv=J, precision=precision, tuning={"grid_walk": g})
           for g in (1, 0)]
    assert ops[0].info()["walk_tasks"] > 0 and ops[1].info()["walk_tasks"] == 0
    oop = oracle_mod.Operator(u, v, None, wt, n, n, 2.0, kernel=kernel, Ju=J, Jv=J)
    y = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    yd = to_dev(torch, y, precision)
    a = to_np(ops[0].adjoint(yd))
    b = to_np(ops[1].adjoint(yd))
    assert rel_l2(a, oop.adjoint(y)) < TOL[precision]
    assert rel_l2(a, b) < (1e-6 if precision == "fp32" else 1e-13)
    assert np.array_equal(a, to_np(ops[0].adjoint(yd)))


def test_column_walk_falls_back_on_full_cells(pg, oracle_mod, cuda):
    """A coverage with more than 256 visibilities on one base cell keeps the
    work items (which split a cell over lanes) even when the walk is asked
    for."""
    torch = cuda
    rng = np.random.default_rng(4)
    M = 5000
    u = rng.normal(0, 10, M)
    v = rng.normal(0, 10, M)
    u[:400] = 0.25
    v[:400] = -0.5
    op = pg.MeasurementOperator(u, v, None, None, 64, 64, 2.0, power_iters=0, kernel="kb", Ju=4,
                                Jv=4, precision="fp32", tuning={"grid_walk": 1})
    assert op.info()["walk_tasks"] == 0
    y = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    oop = oracle_mod.Operator(u, v, None, None, 64, 64, 2.0, kernel="kb", Ju=4, Jv=4)
    assert rel_l2(to_np(op.adjoint(to_dev(torch, y, "fp32"))), oop.adjoint(y)) < TOL["fp32"]


def test_host_entry_points_match_device_path(pg, cuda):
    """The host complex<double> entry points convert and copy in chunks on
    two streams (here 3 chunks of visibilities); their results equal the
    device entry points' on the same FP32-rounded inputs, bit for bit, in
    both directions and on repeated calls."""
    torch = cuda
    rng = np.random.default_rng(17)
    M, n = 700_000, 256
    u, v = rng.normal(0, n / 2, M), rng.normal(0, n / 2, M)
    op = pg.MeasurementOperator(u, v, None, None, n, n, 2.0, power_iters=0, kernel="kb", Ju=4,
                                Jv=4, precision="fp32")
    x = (rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)).astype(np.complex64)
    y = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
    for _ in range(2):
        yh = op.forward(x.astype(np.complex128))
        xh = op.adjoint(y.astype(np.complex128))
        yd = op.forward(torch.from_numpy(x).cuda()).cpu().numpy()
        xd = op.adjoint(torch.from_numpy(y).cuda()).cpu().numpy()
        assert np.array_equal(yh, yd.astype(np.complex128))
        assert np.array_equal(xh, xd.astype(np.complex128))
