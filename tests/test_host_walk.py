"""Column-walk plan of G^H (host, no GPU).

The plan must hold every visibility once, in the walk order the kernel
addresses (per task, per column, per k, the active rows in order), with the
counts and column starts that address it.  A numpy replay of the kernel's
walk (the lanes' sliding J x J blocks, one column flushed per step, four
warps over quarters of the tile's columns, windows added to the grid) must
equal a direct scatter of the same taps: rel. L2 1e-12 (FP64, only the
summation order differs).
"""
import numpy as np
import pytest


def coverage(M, Nu, Nv, seed, spread):
    rng = np.random.default_rng(seed)
    u = rng.normal(0, spread * Nu, M)
    v = rng.normal(0, spread * Nv, M)
    # a few duplicates: several visibilities on one base cell
    u[: M // 10] = u[M // 10: 2 * (M // 10)]
    v[: M // 10] = v[M // 10: 2 * (M // 10)]
    return u, v


def base_cells(u, v, Nu, Nv, J):
    ku, kv = np.floor(u - J / 2), np.floor(v - J / 2)
    q0 = np.mod(ku + 1, Nu).astype(np.int64)
    p0 = np.mod(kv + 1, Nv).astype(np.int64)
    flip = (ku.astype(np.int64) + kv.astype(np.int64)) & 1
    return p0, q0, u - J / 2 - ku, v - J / 2 - kv, flip


def taps(t, J):
    # any smooth tap function: the replay and the direct scatter share it
    j = np.arange(J)
    return np.cos(0.45 * (t[..., None] + J / 2 - j)) + 0.1 * (t[..., None] - 0.3) ** 2


CASES = [(4000, 128, 128, 4, 0.12), (3000, 96, 64, 5, 0.3), (2500, 40, 72, 3, 0.2),
         (1500, 64, 64, 6, 2.0), (5, 64, 64, 4, 0.1)]


@pytest.mark.parametrize("M,Nu,Nv,J,spread", CASES)
def test_walk_plan_structure(pg, M, Nu, Nv, J, spread):
    u, v = coverage(M, Nu, Nv, 3, spread)
    W = pg.WalkPlan(u, v, Nu, Nv, J)
    assert W.M == M
    assert np.array_equal(np.sort(W.slot_user), np.arange(M))
    assert W.win_stride % 2 == 1 and W.win_stride >= W.win_cols
    p0, q0, tu, tv, flip = base_cells(u, v, Nu, Nv, J)
    m = W.slot_user
    assert np.allclose(np.abs(W.frac[:, 0]), tu[m], atol=1e-15)
    assert np.allclose(W.frac[:, 1], tv[m], atol=1e-15)
    assert np.array_equal(np.signbit(W.frac[:, 0]), flip[m] == 1)
    steps = 0
    for k, (P, Q, H, Wd, _, _, tile, _) in enumerate(W.tasks):
        assert W.tile_tasks[tile] == k and W.tile_tasks[tile + 1] == k + 1
        cnt = W.counts[k]
        assert np.all(cnt[Wd:] == 0) and np.all(cnt[:, H:] == 0)
        for q in range(32):
            base = W.colstart[k, q]
            for j in range(int(cnt[q].max(initial=0))):
                rows = np.nonzero(cnt[q] > j)[0]
                s = base + np.arange(rows.size)
                mm = W.slot_user[s]
                assert np.array_equal(p0[mm], P + rows) and np.all(q0[mm] == Q + q)
                for r, x in zip(rows, mm):  # the j-th visibility of the cell, caller order
                    same = np.nonzero((p0 == P + r) & (q0 == Q + q))[0]
                    assert same[j] == x
                base += rows.size
            assert base == W.colstart[k, q + 1]
            steps += int(cnt[q].max(initial=0))
        assert cnt.sum() == W.colstart[k, 32] - W.colstart[k, 0]
    assert steps == W.steps
    assert W.colstart[:, 32].max(initial=0) <= M
    assert sorted(W.task_order) == list(range(len(W.tasks)))


def walk_replay(W, y, nw=4):
    """G^H by the kernel's walk on the plan, windows added to the grid."""
    J, Nu, Nv = W.J, W.Nu, W.Nv
    grid = np.zeros((Nv, Nu), complex)
    lanes = np.arange(32)
    for k, (P, Q, H, Wd, _, _, _, _) in enumerate(W.tasks):
        wins = np.zeros((nw, W.win_rows, W.win_stride), complex)
        for w in range(nw):
            q0, q1 = w * Wd // nw, (w + 1) * Wd // nw
            acc = np.zeros((32, J, J), complex)  # lane, jv, physical column
            if q0 >= q1:
                continue
            for qq in range(q0 - q0 % J, q1 + J - 1, J):
                for p in range(J):
                    q = qq + p
                    if q0 <= q < q1:
                        c = W.counts[k, q]
                        base = W.colstart[k, q]
                        for j in range(int(c.max())):
                            act = c > j
                            s = base + np.cumsum(act)[act] - 1
                            t = W.frac[s]
                            z = np.copysign(1.0, t[:, 0]) * y[W.slot_user[s]]
                            ku, kv = taps(np.abs(t[:, 0]), J), taps(t[:, 1], J)
                            for jv in range(J):
                                for ju in range(J):
                                    acc[lanes[act], jv, (p + ju) % J] += z * kv[:, jv] * ku[:, ju]
                            base += int(act.sum())
                    if q0 <= q < q1 + J - 1:
                        for jv in range(J):
                            wins[w, lanes[:H] + jv, q] += acc[:H, jv, p]
                            acc[:, jv, p] = 0
        win = wins.sum(axis=0)
        rr = (P + np.arange(H + J - 1)) % Nv
        cc = (Q + np.arange(Wd + J - 1)) % Nu
        np.add.at(grid, (rr[:, None], cc[None, :]), win[:H + J - 1, :Wd + J - 1])
    return grid


def direct(u, v, y, Nu, Nv, J):
    p0, q0, tu, tv, flip = base_cells(u, v, Nu, Nv, J)
    ku, kv = taps(tu, J), taps(tv, J)
    z = np.where(flip == 1, -1.0, 1.0) * y
    grid = np.zeros((Nv, Nu), complex)
    for jv in range(J):
        for ju in range(J):
            np.add.at(grid, ((p0 + jv) % Nv, (q0 + ju) % Nu), z * kv[:, jv] * ku[:, ju])
    return grid


@pytest.mark.parametrize("M,Nu,Nv,J,spread", CASES[:4])
def test_walk_replay_matches_direct_scatter(pg, M, Nu, Nv, J, spread):
    u, v = coverage(M, Nu, Nv, 5, spread)
    rng = np.random.default_rng(6)
    y = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    W = pg.WalkPlan(u, v, Nu, Nv, J)
    a, b = walk_replay(W, y), direct(u, v, y, Nu, Nv, J)
    assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(b)


def test_walk_plan_rejects(pg):
    u = np.zeros(4)
    with pytest.raises(pg.PurifyError):
        pg.WalkPlan(u, u, 8, 8, 10)  # support larger than the grid
