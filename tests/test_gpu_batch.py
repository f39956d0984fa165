"""Multi-channel batch against single operators built from the same coverage.

Each channel of a batch must give the result of its own MeasurementOperator
(which the parity tests pin to the FP64 oracle).  The batch runs one grouped
degrid and one grouped grid launch over all channels and a batched cuFFT per
grid size, replayed from a CUDA graph.

Tolerances (relative L2 per channel, batch vs single operator):
  FP64  1e-12
  FP32  2e-6   (cuFFT may pick a different algorithm for a batched plan)
The oracle check of the FP64 batch uses the FP64 bar of the parity tests, 1e-10.
"""
import numpy as np
import pytest

from conftest import rel_l2
from purify_gb300 import synthetic

pytestmark = pytest.mark.gpu

TOL = {"fp32": 2e-6, "fp64": 1e-12}
TUNING = {"tile": 32, "max_per_item": 16, "degrid_threads": 128, "grid_threads": 128}


def channels_small(seed=3):
    """Six channels: three image sizes (one non-square), uneven visibility
    counts, one empty channel and one with complex weights."""
    rng = np.random.default_rng(seed)
    sizes = [(64, 64), (128, 128), (64, 64), (96, 128), (128, 128), (64, 64)]
    Ms = [3000, 20000, 0, 12000, 7000, 1]
    chans = []
    for k, ((ny, nx), M) in enumerate(zip(sizes, Ms)):
        u, v = synthetic.gaussian_core_uv(M, 2 * nx, 2 * ny, 0.25, seed=seed + k, scale=1 + 0.01 * k)
        ch = dict(u=u, v=v, imsizey=ny, imsizex=nx)
        if k == 4:
            ch["weights"] = rng.standard_normal(M) + 1j * rng.standard_normal(M)
        chans.append(ch)
    return chans


def dev(torch, a, precision):
    dt = torch.complex64 if precision == "fp32" else torch.complex128
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128)).to(dtype=dt).cuda()


def host(t):
    return t.cpu().numpy().astype(np.complex128)


def single_ops(pg, chans, precision, threads=128, tile=32, max_per_item=16):
    return [pg.MeasurementOperator(c["u"], c["v"], None, c.get("weights"), c["imsizey"],
                                   c["imsizex"], 2.0, power_iters=0, kernel="kb", Ju=4, Jv=4,
                                   precision=precision,
                                   tuning={"threads": threads, "tile": tile,
                                           "max_per_item": max_per_item, "fused_permute": -1})
            for c in chans]


def inputs(torch, chans, precision, seed=11):
    xs, ys = [], []
    for k, c in enumerate(chans):
        xs.append(dev(torch, synthetic.sky_image(c["imsizey"], c["imsizex"], seed=seed + k),
                      precision))
        ys.append(dev(torch, synthetic.random_vis(c["u"].size, seed=seed + 100 + k), precision))
    return xs, ys


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_matches_single_operators(pg, cuda, precision):
    torch = cuda
    chans = channels_small()
    b = pg.Batch(chans, J=4, precision=precision, tuning=TUNING)
    ops = single_ops(pg, chans, precision)
    xs, ys = inputs(torch, chans, precision)
    vis = [torch.empty(c["u"].size, dtype=b.complex_dtype, device="cuda") for c in chans]
    xo = [torch.empty_like(x) for x in xs]
    b.bind(xs, vis, xo)
    b.apply(1)
    torch.cuda.synchronize()
    for k, op in enumerate(ops):
        ref = host(op.forward(xs[k]))
        got = host(vis[k])
        if ref.size:
            assert rel_l2(got, ref) < TOL[precision], k
    # adjoint from independent visibilities
    b.bind(xs, ys, xo)
    b.apply(2)
    torch.cuda.synchronize()
    for k, op in enumerate(ops):
        ref = host(op.adjoint(ys[k]))
        got = host(xo[k])
        if chans[k]["u"].size:
            assert rel_l2(got, ref) < TOL[precision], k
        else:
            assert np.all(got == 0)


def test_batch_fp64_matches_oracle(pg, oracle_mod, cuda):
    torch = cuda
    chans = channels_small()
    b = pg.Batch(chans, J=4, precision="fp64", tuning=TUNING)
    xs, ys = inputs(torch, chans, "fp64")
    vis = [torch.empty(c["u"].size, dtype=b.complex_dtype, device="cuda") for c in chans]
    xo = [torch.empty_like(x) for x in xs]
    b.bind(xs, vis, xo)
    b.apply(1)
    torch.cuda.synchronize()
    for k, c in enumerate(chans):
        if c["u"].size < 2:
            continue
        oop = oracle_mod.Operator(c["u"], c["v"], None, c.get("weights"), c["imsizey"],
                                  c["imsizex"], 2.0, kernel="kb", Ju=4, Jv=4)
        assert rel_l2(host(vis[k]), oop.forward(host(xs[k]))) < 1e-10, k


def test_batch_both_directions_and_rebind(pg, cuda):
    """directions=3 is Phi^H Phi; a rebind switches buffers without a new
    recording; replays are bit-identical."""
    torch = cuda
    precision = "fp32"
    chans = channels_small()
    b = pg.Batch(chans, J=4, precision=precision, tuning=TUNING)
    xs, _ = inputs(torch, chans, precision)
    xs2, _ = inputs(torch, chans, precision, seed=77)
    vis = [torch.empty(c["u"].size, dtype=b.complex_dtype, device="cuda") for c in chans]
    xo = [torch.empty_like(x) for x in xs]
    b.bind(xs, vis, xo)
    b.apply(3)
    torch.cuda.synchronize()
    first = [host(t) for t in xo]
    b.apply(3)
    torch.cuda.synchronize()
    for k in range(len(chans)):
        assert np.array_equal(host(xo[k]), first[k]), k
    ops = single_ops(pg, chans, precision)
    for k, op in enumerate(ops):
        ref = host(op.adjoint(op.forward(xs[k])))
        if chans[k]["u"].size:
            assert rel_l2(first[k], ref) < TOL[precision], k
    # rebind to other inputs and outputs
    xo2 = [torch.empty_like(x) for x in xs]
    b.bind(xs2, vis, xo2)
    b.apply(3)
    torch.cuda.synchronize()
    for k, op in enumerate(ops):
        ref = host(op.adjoint(op.forward(xs2[k])))
        if chans[k]["u"].size:
            assert rel_l2(host(xo2[k]), ref) < TOL[precision], k
    # the first outputs were not touched by the rebound replay
    for k in range(len(chans)):
        assert np.array_equal(host(xo[k]), first[k]), k


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_power_method(pg, cuda, precision):
    """Per-channel norms follow each channel's own stopping step: they match
    single operators' power methods, and a channel's norm does not depend on
    the other channels of the batch."""
    torch = cuda
    chans = [c for c in channels_small() if c["u"].size > 0]
    b = pg.Batch(chans, J=4, precision=precision, tuning=TUNING)
    norms = b.power_method(60, 1e-4)
    assert np.allclose(b.norms, norms, rtol=0, atol=0)
    ops = single_ops(pg, chans, precision)
    ref = np.array([op.power_method(60, 1e-4) for op in ops])
    tol = 1e-5 if precision == "fp32" else 1e-12
    assert np.max(np.abs(norms - ref) / ref) < tol
    # the same channel alone
    alone = pg.Batch(chans[1:2], J=4, precision=precision, tuning=TUNING)
    n1 = alone.power_method(60, 1e-4)
    assert abs(n1[0] - norms[1]) / norms[1] < tol
    # applies after the power method divide by the norms
    xs, _ = inputs(torch, chans, precision)
    vis = [torch.empty(c["u"].size, dtype=b.complex_dtype, device="cuda") for c in chans]
    b.bind(xs, vis, None)
    b.apply(1)
    torch.cuda.synchronize()
    for k, op in enumerate(ops):
        assert rel_l2(host(vis[k]), host(op.forward(xs[k]))) < max(tol, TOL[precision]) * 10, k


def test_batch_autotuned(pg, cuda):
    torch = cuda
    chans = channels_small()
    b = pg.Batch(chans, J=4, precision="fp32")
    t = b.tuning
    assert t["tile"] in (24, 32, 48)
    assert t["degrid_threads"] in (64, 128, 256) and t["grid_threads"] in (64, 128, 256)
    info = b.info()
    assert info["channels"] == len(chans)
    assert info["visibilities"] == sum(c["u"].size for c in chans)
    assert info["size_groups"] == 3
    ops = single_ops(pg, chans, "fp32", threads=128, tile=t["tile"],
                     max_per_item=t["max_per_item"])
    xs, ys = inputs(torch, chans, "fp32")
    vis = [torch.empty(c["u"].size, dtype=b.complex_dtype, device="cuda") for c in chans]
    xo = [torch.empty_like(x) for x in xs]
    b.bind(xs, vis, xo)
    b.apply(1)
    torch.cuda.synchronize()
    for k, op in enumerate(ops):
        if chans[k]["u"].size:
            assert rel_l2(host(vis[k]), host(op.forward(xs[k]))) < TOL["fp32"], k


def test_batch_errors(pg, cuda):
    chans = channels_small()[:2]
    b = pg.Batch(chans, J=4, precision="fp32", tuning=TUNING)
    with pytest.raises(pg.PurifyError):
        b.apply(1)  # nothing bound
    with pytest.raises(pg.PurifyError):
        b.apply(4)
    with pytest.raises(pg.PurifyError):
        b.set_norms([1.0, 0.0])
    with pytest.raises(pg.PurifyError):
        pg.Batch([], J=4)
    with pytest.raises(pg.PurifyError):
        pg.Batch([dict(u=np.zeros(3), v=np.zeros(3), imsizey=0, imsizex=8)], J=4, tuning=TUNING)


@pytest.mark.parametrize("J", [2, 6])
def test_batch_weights_any_kernel_fit(pg, cuda, J):
    """Channels with complex weights, for a sub-segmented tap fit (KB J = 2)
    and a plain one (J = 6): the grouped launches apply the weights around
    the gridding kernels (caller order after G, conjugated by the gather
    before G^H), as the single operator does."""
    torch = cuda
    rng = np.random.default_rng(J)
    chans = []
    for k, M in enumerate((3000, 5000)):
        chans.append(dict(u=rng.normal(0, 12, M), v=rng.normal(0, 12, M), imsizey=48, imsizex=48,
                          weights=rng.standard_normal(M) + 1j * rng.standard_normal(M)))
    b = pg.Batch(chans, J=J, precision="fp32", tuning=TUNING)
    ops = [pg.MeasurementOperator(c["u"], c["v"], None, c["weights"], 48, 48, 2.0, power_iters=0,
                                  kernel="kb", Ju=J, Jv=J, precision="fp32",
                                  tuning={"threads": 128, "tile": 32, "max_per_item": 16})
           for c in chans]
    xs = [dev(torch, rng.standard_normal(48 * 48) + 1j * rng.standard_normal(48 * 48), "fp32")
          for _ in chans]
    vis = [torch.empty(c["u"].size, dtype=torch.complex64, device="cuda") for c in chans]
    xo = [torch.empty(48 * 48, dtype=torch.complex64, device="cuda") for _ in chans]
    b.bind(xs, vis, xo)
    b.apply(3)
    torch.cuda.synchronize()
    for k, op in enumerate(ops):
        y = op.forward(xs[k])
        assert rel_l2(host(vis[k]), host(y)) < TOL["fp32"], k
        assert rel_l2(host(xo[k]), host(op.adjoint(vis[k]))) < TOL["fp32"], k


def test_fused_and_unfused_size_groups(pg, cuda):
    """FP32 size groups of a power-of-two grid width run as interleaved grids
    (one row-pass launch and one column plan per group); the others (here a
    192-wide grid) keep the padded 2-D transform.  A batch mixing both must
    still match every channel's own operator."""
    torch = cuda
    chans = []
    for k, ((ny, nx), M) in enumerate(zip([(64, 64), (64, 96), (64, 64), (32, 96), (64, 64)],
                                          [4000, 5000, 3000, 2000, 0])):
        u, v = synthetic.gaussian_core_uv(M, 2 * nx, 2 * ny, 0.25, seed=40 + k)
        chans.append(dict(u=u, v=v, imsizey=ny, imsizex=nx))
    b = pg.Batch(chans, J=4, precision="fp32", tuning=TUNING)
    assert b.info()["size_groups"] == 3
    ops = single_ops(pg, chans, "fp32")
    xs, ys = inputs(torch, chans, "fp32", seed=5)
    vis = [torch.empty(c["u"].size, dtype=b.complex_dtype, device="cuda") for c in chans]
    xo = [torch.empty_like(x) for x in xs]
    b.bind(xs, vis, xo)
    for _ in range(2):  # the padded grids keep their zero rows between applies
        b.apply(1)
    b.bind(xs, ys, xo)
    b.apply(2)
    torch.cuda.synchronize()
    for k, op in enumerate(ops):
        if chans[k]["u"].size:
            assert rel_l2(host(vis[k]), host(op.forward(xs[k]))) < TOL["fp32"], k
            assert rel_l2(host(xo[k]), host(op.adjoint(ys[k]))) < TOL["fp32"], k
        else:
            assert np.all(host(xo[k]) == 0)
