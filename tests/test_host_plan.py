"""Host logic of the GB300 operator on the CPU: tap-weight polynomials and the
coverage plan.  The plan is replayed in numpy exactly as the device kernels
consume it (windows, work items, tasks, fold order) and compared with the
oracle's explicit CSR G and G^H (operators.cc:8-46, operators.h:123-145)."""
import numpy as np
import pytest

from conftest import rel_l2

KERNEL_CASES = [("kb", J) for J in range(1, 9)] + [
    ("pswf", 6), ("gauss", 4), ("gauss", 6), ("box", 3), ("kbmin", 4), ("gauss_alt", 5)]


@pytest.mark.parametrize("kernel,J", KERNEL_CASES)
def test_tap_polynomials_match_kernel(pg, oracle_mod, kernel, J):
    t = np.random.default_rng(J).random(4001)
    t[:3] = [0.0, 0.5, np.nextafter(1.0, 0.0)]
    j = np.arange(J)
    args = t[:, None] + J / 2.0 - 1.0 - j[None, :]
    exact = oracle_mod.kernel_values(kernel, J, args.ravel()).reshape(args.shape)
    exact *= np.where(j % 2 == 1, -1.0, 1.0)[None, :]
    peak = np.abs(exact).max()
    f64, e64 = pg.kernel_taps(kernel, J, t, precision="fp64")
    f32, e32 = pg.kernel_taps(kernel, J, t, precision="fp32")
    assert np.abs(f64 - exact).max() <= 1e-12 * peak, (e64, np.abs(f64 - exact).max())
    # FP32: the fit is within 3e-8 of the kernel; Horner in FP32 adds rounding.
    assert np.abs(f32 - exact).max() <= 3e-7 * peak, (e32, np.abs(f32 - exact).max())


def _lanes(plan, b):
    base, kmax = plan.batches[b]
    for lane in range(32):
        code = int(plan.lane_code[b, lane])
        lp, lq, cnt = code & 0xFF, (code >> 8) & 0xFF, (code >> 16) & 0xFFFF
        yield lane, lp, lq, cnt, [base + 32 * k + lane for k in range(kmax)]


def group_uv(group):
    """Cells of a work item along u and v: 1 x 1, 2 x 2, or a pair of a row."""
    return (1 if group == 1 else 2), (2 if group == 2 else 1)


def block_taps(plan, kernel="kb"):
    """Tap vectors of every slot over its item's register block (J + g - 1
    cells along an axis where the item spans g cells): the J taps at the
    fraction's cell d inside the group (frac = t + d), zeros elsewhere — what
    block_taps evaluates on the device."""
    import purify_gb300 as pg
    J = plan.J
    out = []
    for axis, G in zip((0, 1), group_uv(plan.group)):
        f = plan.frac[:, axis]
        d = np.floor(f).astype(int) if G == 2 else np.zeros(f.size, dtype=int)
        assert d.min() >= 0 and d.max() <= G - 1
        taps, _ = pg.kernel_taps(kernel, J, f - d, precision="fp64")
        blk = np.zeros((f.size, J + G - 1))
        for k in range(G):
            sel = d == k
            blk[sel, k:k + J] = taps[sel]
        out.append(blk)
    return out


def replay_degrid(plan, taps_u, taps_v, grid):
    """Slot values as degrid_kernel writes them, then compact_kernel."""
    gu, gv = group_uv(plan.group)
    JBU, JBV, Nu, Nv = plan.J + gu - 1, plan.J + gv - 1, plan.Nu, plan.Nv
    slots = np.zeros(plan.S, dtype=np.complex128)
    g = grid.reshape(Nv, Nu)
    for (P, Q, H, W, b0, b1, tile, _) in plan.tasks:
        for b in range(b0, b1):
            for lane, lp, lq, cnt, sl in _lanes(plan, b):
                assert lp < H and lq < W
                assert lp % gv == 0 and lq % gu == 0
                rows = (P + lp + np.arange(JBV)) % Nv
                cols = (Q + lq + np.arange(JBU)) % Nu
                F = g[np.ix_(rows, cols)]
                for k, i in enumerate(sl):
                    assert (plan.slot_user[i] >= 0) == (k < cnt)
                    slots[i] = plan.weight[i] * (taps_v[i] @ F @ taps_u[i])
    return slots[plan.user_slot]


def replay_grid(plan, taps_u, taps_v, vis):
    """expand_kernel, task windows as grid_kernel writes them, then
    fold_kernel's fixed-order sum."""
    gu, gv = group_uv(plan.group)
    JU, JV, Nu, Nv = plan.J + gu - 1, plan.J + gv - 1, plan.Nu, plan.Nv  # the block's extent
    slots = np.where(plan.slot_user >= 0, vis[np.maximum(plan.slot_user, 0)], 0)
    windows = []
    for (P, Q, H, W, b0, b1, tile, _) in plan.tasks:
        win = np.zeros((H + JV - 1, W + JU - 1), dtype=np.complex128)
        for b in range(b0, b1):
            cells = set()
            for lane, lp, lq, cnt, sl in _lanes(plan, b):
                if cnt == 0:
                    continue
                assert (lp, lq) not in cells, "two items of one base cell in a batch"
                cells.add((lp, lq))
                for i in sl:
                    z = np.conj(plan.weight[i]) * slots[i]
                    win[lp:lp + JV, lq:lq + JU] += z * np.outer(taps_v[i], taps_u[i])
        windows.append(win)
    ntu, ntv = plan.ntu, plan.ntv
    grid = np.zeros((Nv, Nu), dtype=np.complex128)
    tu, tv = plan.tu_start, plan.tv_start
    for p in range(Nv):
        a = np.searchsorted(tv, p, side="right") - 1
        for q in range(Nu):
            b = np.searchsorted(tu, q, side="right") - 1
            lp, lq = p - tv[a], q - tu[b]
            a2, b2 = (a - 1) % ntv, (b - 1) % ntu
            hp, wp = tv[a2 + 1] - tv[a2], tu[b2 + 1] - tu[b2]
            s = 0j
            for (ta, tb, r, c, on) in ((a, b, lp, lq, True), (a2, b, lp + hp, lq, lp < JV - 1),
                                       (a, b2, lp, lq + wp, lq < JU - 1),
                                       (a2, b2, lp + hp, lq + wp, lp < JV - 1 and lq < JU - 1)):
                if not on:
                    continue
                t = ta * ntu + tb
                for k in range(plan.tile_tasks[t], plan.tile_tasks[t + 1]):
                    s += windows[k][r, c]
            grid[p, q] = s
    return grid.ravel()


@pytest.mark.parametrize("n,J,M,spread,seed,group", [
    (16, 4, 10, 1.0, 0, 1),     # the reference's golden operator shape
    (24, 6, 300, 12.0, 1, 1),   # grid 48: two uneven tiles per axis
    (40, 3, 500, 40.0, 2, 1),   # u, v well outside the grid: periodic wrap
    (20, 8, 200, 3.0, 3, 1),    # dense: many visibilities per cell, several layers
    (18, 5, 64, 9.0, 4, 1),     # odd support, 36-cell grid
    (16, 4, 10, 1.0, 0, 2),     # 2 x 2 cell groups: the same shapes
    (24, 6, 300, 12.0, 1, 2),
    (40, 3, 500, 40.0, 2, 2),
    (20, 5, 200, 3.0, 3, 2),
    (18, 5, 64, 9.0, 4, 2),     # 36-cell grid: tiles of 18, odd halo
    (25, 2, 400, 8.0, 5, 2),    # odd grid width (50): tiles of 25, a last group of one cell
    (16, 4, 10, 1.0, 0, 3),     # pairs of cells of a row
    (25, 2, 400, 8.0, 5, 3),    # pairs, odd tile width: a last pair of one cell
    (48, 6, 3000, 20.0, 2, 3),
])
def test_plan_replay_matches_oracle_G(pg, oracle_mod, n, J, M, spread, seed, group):
    rng = np.random.default_rng(seed)
    u = rng.normal(0, spread, M)
    v = rng.normal(0, spread, M)
    wt = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    Nu = Nv = 2 * n
    plan = pg.CoveragePlan(u, v, Nu, Nv, J, weights=wt, group=group)
    assert plan.group == group and not plan.unit_weights
    assert sorted(plan.user_slot.tolist()) == sorted(np.flatnonzero(plan.slot_user >= 0).tolist())
    assert np.array_equal(plan.slot_user[plan.user_slot], np.arange(M))
    taps_u, taps_v = block_taps(plan)
    op = oracle_mod.Operator(u, v, None, wt, n, n, 2.0, kernel="kb", Ju=J, Jv=J)
    grid = rng.standard_normal(Nu * Nv) + 1j * rng.standard_normal(Nu * Nv)
    y = replay_degrid(plan, taps_u, taps_v, grid)
    assert rel_l2(y, op.G_forward(grid)) < 1e-12
    vis = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    g = replay_grid(plan, taps_u, taps_v, vis)
    assert rel_l2(g, op.G_adjoint(vis)) < 1e-12


def test_unit_weights_plan_matches_oracle(pg, oracle_mod):
    rng = np.random.default_rng(8)
    M, n, J = 400, 24, 4
    u = rng.normal(0, 10, M)
    v = rng.normal(0, 10, M)
    plan = pg.CoveragePlan(u, v, 2 * n, 2 * n, J)
    assert plan.unit_weights
    taps_u, taps_v = block_taps(plan)
    op = oracle_mod.Operator(u, v, None, None, n, n, 2.0, kernel="kb", Ju=J, Jv=J)
    grid = rng.standard_normal(4 * n * n) + 1j * rng.standard_normal(4 * n * n)
    assert rel_l2(replay_degrid(plan, taps_u, taps_v, grid), op.G_forward(grid)) < 1e-12
    vis = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    assert rel_l2(replay_grid(plan, taps_u, taps_v, vis), op.G_adjoint(vis)) < 1e-12


def test_plan_empty_and_bad_sizes(pg):
    p = pg.CoveragePlan(np.zeros(0), np.zeros(0), 32, 32, 4)
    assert p.M == 0 and p.S == 0 and p.batches.shape[0] == 0
    with pytest.raises(pg.PurifyError):
        pg.CoveragePlan(np.zeros(3), np.zeros(3), 4, 4, 6)  # grid smaller than the support


def test_plan_balances_dense_cells(pg):
    # 5000 visibilities in one cell: split into items of <= 16, one per layer
    u = np.full(5000, 0.25)
    v = np.full(5000, -0.5)
    p = pg.CoveragePlan(u, v, 64, 64, 4)
    counts = (p.lane_code >> 16) & 0xFFFF
    assert counts.sum() == 5000 and counts.max() <= 16
    assert (p.slot_user >= 0).sum() == 5000


@pytest.mark.parametrize("group", [1, 2, 3])
def test_batch_lanes_are_bank_classes(pg, group):
    """Items sit on the lane of their bank class (window offset lp * stride +
    lq = lane, mod 16) wherever that lane was free, so half-warps mostly touch
    distinct shared-memory bank pairs at each tap offset; the stride is the
    widest window.  A batch holds at most 4 items of a class, spread over the
    two half-warps, and its items of the leading count at most 2, so a
    half-warp's lane-block access mostly costs one or two wavefronts.  With
    2 x 2 cell groups the anchors sit on even rows and columns; the window's
    extra cell per two rows keeps their offsets on all 16 classes."""
    from purify_gb300 import synthetic
    u, v = synthetic.mixed_uv(200_000, 512, 512, 0.7, 0.15, seed=3)
    p = pg.CoveragePlan(u, v, 512, 512, 6, group=group)
    lc = p.lane_code
    lp, lq, cnt = lc & 0xFF, (lc >> 8) & 0xFF, lc >> 16
    # window offset of the item's anchor (one extra cell per two rows with
    # 2 x 2 groups, whose anchors sit on even rows and columns)
    r = (lp * p.win_stride + lq + (lp >> 1) * (group == 2)) & 15
    lane = np.arange(32)[None, :] & 15
    valid = cnt > 0
    on_class = ((r == lane) & valid).sum() / valid.sum()
    assert on_class > (0.8 if group == 1 else 0.7)
    assert valid.mean() > 0.9
    per_batch, per_half = [], []
    for b in range(lc.shape[0]):
        per_batch.append(np.bincount(r[b][valid[b]], minlength=16).max())
        for h in range(2):
            sel = slice(16 * h, 16 * h + 16)
            if valid[b][sel].any():
                per_half.append(np.bincount(r[b][sel][valid[b][sel]], minlength=16).max())
    assert max(per_batch) <= 4
    # single cells: 1.6 per half-warp; 2 x 2 groups, with fewer items per
    # tile to pack: 2.0 (their anchors still cover all 16 classes)
    assert np.mean(per_half) < (1.8 if group == 1 else 2.1)
    assert len(np.unique(r[valid])) == 16


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_plan_rejects_non_finite_coordinates(pg, bad):
    u = np.zeros(10)
    v = np.zeros(10)
    u[3] = bad
    with pytest.raises(pg.PurifyError) as e:
        pg.CoveragePlan(u, v, 64, 64, 4)
    assert e.value.status == 1
    with pytest.raises(pg.PurifyError):
        pg.CoveragePlan(v, u, 64, 64, 4)


def _warp_efficiency(plan, nw, order=None):
    """Mean over tasks of (mean warp load / largest warp load) when batch i of
    a task goes to warp i mod nw; a batch costs 220 per k-step plus 180 (the
    planner's model).  `order` re-sorts each task's batches first."""
    kmax = plan.batches[:, 1].astype(np.int64)
    eff = []
    for t in plan.tasks:
        cost = 220.0 * kmax[t[4]:t[5]] + 180.0
        if order is not None:
            cost = order(cost)
        loads = np.zeros(nw)
        for i, c in enumerate(cost):
            loads[i % nw] += c
        eff.append(cost.sum() / nw / loads.max())
    return float(np.mean(eff))


def test_task_batches_balanced_over_warps(pg):
    """The planner orders each task's batches (default: 4 warps) so that
    round-robin dealing balances the warps better than the heaviest-first
    order, and the reordering keeps every batch and every slot."""
    rng = np.random.default_rng(21)
    M, N = 300_000, 512
    u = np.concatenate([rng.normal(0, 0.08 * N, M // 2), rng.uniform(-N / 2, N / 2, M - M // 2)])
    v = np.concatenate([rng.normal(0, 0.08 * N, M // 2), rng.uniform(-N / 2, N / 2, M - M // 2)])
    plan = pg.CoveragePlan(u, v, N, N, 6)
    balanced = _warp_efficiency(plan, 4)
    heaviest_first = _warp_efficiency(plan, 4, order=lambda c: np.sort(c)[::-1])
    assert balanced >= 0.9 and balanced > heaviest_first + 0.05, (balanced, heaviest_first)
    # every slot of every batch is a distinct slot of the plan
    slots = np.concatenate([b + 32 * np.arange(k)[:, None] + np.arange(32)[None, :]
                            for b, k in plan.batches], axis=None)
    assert slots.size == plan.S and np.unique(slots).size == plan.S
