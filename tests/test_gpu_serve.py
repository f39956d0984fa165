"""Request server: results alone and in a concurrent mix, admission by the
HBM budget, norm requests.

A request owns its workspace and runs the same kernels with the same plans
as a single operator, so its result is bit-identical alone, in a mix and
through the operator's host entry points: the tolerance here is 0 (exact
equality).  Norm requests follow the single-operator power method and
return the same estimate.
"""
import numpy as np
import pytest

from purify_gb300 import synthetic

pytestmark = pytest.mark.gpu


def coverages(seed=5):
    out = []
    for k, (ny, nx, M, prec) in enumerate([(64, 64, 4000, "fp32"), (128, 128, 30000, "fp32"),
                                            (96, 128, 12000, "fp32"), (64, 64, 5000, "fp64")]):
        u, v = synthetic.gaussian_core_uv(M, 2 * nx, 2 * ny, 0.25, seed=seed + k)
        out.append(dict(u=u, v=v, imsizey=ny, imsizex=nx, precision=prec))
    return out


def add_all(srv, covs, power_iters=20):
    return [srv.add_coverage(c["u"], c["v"], None, None, c["imsizey"], c["imsizex"],
                             power_iters=power_iters, precision=c["precision"]) for c in covs]


def requests(covs, ids, n=24, seed=9):
    rng = np.random.default_rng(seed)
    kinds = ["forward_adjoint", "adjoint", "forward", "norm"]
    out = []
    for r in range(n):
        k = int(rng.integers(len(ids)))
        c = covs[k]
        kind = kinds[r % len(kinds)]
        x = synthetic.sky_image(c["imsizey"], c["imsizex"], seed=seed + r)
        vis = synthetic.random_vis(c["u"].size, seed=seed + 100 + r)
        out.append(dict(coverage=ids[k], kind=kind, x=x, vis=vis, iters=15))
    return out


def run_mix(srv, reqs):
    tickets = [srv.submit(q["coverage"], q["kind"], q["x"], q["vis"], q["iters"]) for q in reqs]
    return [srv.wait(t) for t in tickets]


def same(a, b):
    for key in ("vis", "x"):
        assert (key in a) == (key in b)
        if key in a:
            assert np.array_equal(a[key], b[key]), key
    assert a["norm"] == b["norm"] and a["iterations"] == b["iterations"]


def test_alone_equals_mix(pg, cuda):
    covs = coverages()
    srv = pg.Server(slots=6, hbm_budget=4 << 30)
    ids = add_all(srv, covs)
    reqs = requests(covs, ids)
    mix = run_mix(srv, reqs)
    assert all(r["status"] == 0 for r in mix)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["inflight_peak"] > 1
    for q, m in zip(reqs, mix):
        alone = srv.wait(srv.submit(q["coverage"], q["kind"], q["x"], q["vis"], q["iters"]))
        same(alone, m)


def test_matches_single_operator(pg, cuda):
    covs = coverages()
    srv = pg.Server(slots=4, hbm_budget=2 << 30)
    ids = add_all(srv, covs, power_iters=20)
    for c, cid in zip(covs, ids):
        op = pg.MeasurementOperator(c["u"], c["v"], None, None, c["imsizey"], c["imsizex"], 2.0,
                                    power_iters=20, precision=c["precision"])
        x = synthetic.sky_image(c["imsizey"], c["imsizex"], seed=1)
        vis = synthetic.random_vis(c["u"].size, seed=2)
        r = srv.wait(srv.submit(cid, "forward_adjoint", x))
        y = op.forward(x)
        assert np.array_equal(r["vis"], y)
        assert np.array_equal(r["x"], op.adjoint(y))
        r = srv.wait(srv.submit(cid, "adjoint", vis=vis))
        assert np.array_equal(r["x"], op.adjoint(vis))
        r = srv.wait(srv.submit(cid, "norm", iters=30, tol=1e-4))
        assert r["status"] == 0
        assert r["norm"] == op.power_method(30, 1e-4)


def test_admission_by_budget(pg, cuda):
    covs = coverages()[:2]
    probe = pg.Server(slots=8, hbm_budget=1 << 40)
    ids = add_all(probe, covs, power_iters=0)
    need = max(probe.request_bytes(ids[1], "forward_adjoint"), probe.request_bytes(ids[0], "norm"))
    probe.close()
    budget = int(need * 1.5)  # room for one large request at a time
    srv = pg.Server(slots=8, hbm_budget=budget)
    ids = add_all(srv, covs, power_iters=0)
    reqs = requests(covs, ids, n=16)
    res = run_mix(srv, reqs)
    assert all(r["status"] == 0 for r in res)
    st = srv.stats()
    assert st["bytes_peak"] <= budget
    assert st["completed"] == 16
    # a request that can never fit is refused, not queued
    tiny = pg.Server(slots=2, hbm_budget=1 << 20)
    tid = add_all(tiny, covs[1:2], power_iters=0)[0]
    r = tiny.wait(tiny.submit(tid, "forward_adjoint", synthetic.sky_image(128, 128)))
    assert r["status"] == 6  # REJECTED
    assert tiny.stats()["rejected"] == 1


def test_request_errors(pg, cuda):
    srv = pg.Server(slots=2, hbm_budget=1 << 30)
    cid = add_all(srv, coverages()[:1], power_iters=0)[0]
    with pytest.raises(pg.PurifyError):
        srv.submit(cid, "forward", np.zeros(10))  # wrong image size
    with pytest.raises(pg.PurifyError):
        srv.submit(cid + 5, "norm")  # unknown coverage
    with pytest.raises(pg.PurifyError):
        srv.wait(123456)  # unknown ticket
    with pytest.raises(pg.PurifyError):
        pg.Server(slots=0)


def test_w_projection_coverage(pg, cuda):
    """A w-projection coverage served: the same result as the operator's host
    entry points (the server runs the same row kernels on its workspace)."""
    rng = np.random.default_rng(8)
    n, M = 64, 3000
    u = rng.normal(0, 16, M)
    v = rng.normal(0, 16, M)
    du = 60.0 * 60.0 * 180.0 / 1.0 / (2 * n) / np.pi
    w = rng.uniform(-12 * du, 12 * du, M)
    srv = pg.Server(slots=2, hbm_budget=1 << 30)
    cid = srv.add_coverage(u, v, w, None, n, n, power_iters=5, w_term=True, Jw=6,
                           precision="fp32")
    op = pg.MeasurementOperator(u, v, w, None, n, n, 2.0, power_iters=5, w_term=True, Jw=6,
                                precision="fp32")
    x = synthetic.sky_image(n, n, seed=3)
    r = srv.wait(srv.submit(cid, "forward_adjoint", x))
    y = op.forward(x)
    assert np.array_equal(r["vis"], y)
    assert np.array_equal(r["x"], op.adjoint(y))
    r = srv.wait(srv.submit(cid, "norm", iters=10, tol=0.0))
    assert r["norm"] == op.power_method(10, 0.0)


def test_norm_slots_and_priorities(pg, cuda):
    """Norm requests hold at most norm_slots slots (low stream priority);
    short requests take the high-priority slots first, else any free slot.
    A mix submitted in one burst completes, each result equal to the same
    request alone; norm_slots outside [0, slots] is refused."""
    covs = coverages()
    srv = pg.Server(slots=4, hbm_budget=4 << 30, norm_slots=1)
    ids = add_all(srv, covs)
    reqs = requests(covs, ids, n=20, seed=21)
    # the norms first, so short requests pass norms that wait for the one long slot
    reqs.sort(key=lambda q: q["kind"] != "norm")
    mix = run_mix(srv, reqs)
    assert all(r["status"] == 0 for r in mix)
    assert srv.stats()["completed"] == len(reqs)
    for q, m in zip(reqs, mix):
        same(srv.wait(srv.submit(q["coverage"], q["kind"], q["x"], q["vis"], q["iters"])), m)
    with pytest.raises(pg.PurifyError):
        pg.Server(slots=2, norm_slots=3)
