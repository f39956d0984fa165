"""Coverage ingest on the CPU: the .vis reader against the oracle's
restatement of utilities::read_visibility (utilities.cc:140-188) on rows of
the reference's own PADMM coverage (tests/golden/padmm_input_head.vis) and on
w-term / nan / inf files; the device-free weightings of init_weights."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

VIS = os.path.join(GOLDEN, "padmm_input_head.vis")


def test_read_visibility_matches_oracle(pg, oracle_mod):
    got = pg.read_visibility(VIS)
    ref = oracle_mod.read_visibility(VIS)
    assert got["u"].size == 400
    for k in ("u", "v", "vis", "weights"):
        assert np.array_equal(got[k], ref[k]), k
    # the v reflection of utilities.cc:178
    first = open(VIS).readline().split()
    assert got["v"][0] == -float(first[1])


def test_read_visibility_w_term_and_specials(pg, oracle_mod, tmp_path):
    rng = np.random.default_rng(2)
    rows = rng.standard_normal((50, 6))
    rows[:, 5] = np.abs(rows[:, 5]) + 0.1
    p = tmp_path / "w.vis"
    with open(p, "w") as f:
        for r in rows:
            f.write(" ".join("%.13g" % x for x in r) + "\n")
        f.write("1 2 3 nan inf 0.5\n")
    got = pg.read_visibility(str(p), w_term=True)
    ref = oracle_mod.read_visibility(str(p), w_term=True)
    for k in ("u", "v", "w", "weights"):
        assert np.array_equal(got[k], ref[k]), k
    assert np.array_equal(got["vis"], ref["vis"], equal_nan=True)
    assert np.isnan(got["vis"][-1].real) and np.isinf(got["vis"][-1].imag)


def test_read_visibility_errors(pg, tmp_path):
    with pytest.raises(pg.PurifyError):
        pg.read_visibility(str(tmp_path / "missing.vis"))
    p = tmp_path / "bad.vis"
    p.write_text("1 2 3 4\n")
    with pytest.raises(pg.PurifyError):
        pg.read_visibility(str(p))
    p.write_text("1 2 x 4 5\n")
    with pytest.raises(pg.PurifyError):
        pg.read_visibility(str(p))


@pytest.mark.parametrize("kind", ["none", "natural", "whiten"])
def test_host_weightings(pg, oracle_mod, kind):
    d = pg.read_visibility(VIS)
    got = pg.init_weights(d["u"], d["v"], d["weights"], 2.0, kind, 0.0, 64, 64)
    ref = oracle_mod.init_weights(d["u"], d["v"], d["weights"], 2.0, kind, 0.0, 64, 64)
    assert np.array_equal(got, ref)
    with pytest.raises(pg.PurifyError):
        pg.init_weights(d["u"], d["v"], d["weights"], 2.0, 9, 0.0, 64, 64)


def test_weights_reject_non_finite(pg):
    u = np.zeros(5)
    u[2] = np.nan
    with pytest.raises(pg.PurifyError):
        pg.init_weights(u, np.zeros(5), np.ones(5), 2.0, "uniform", 0.0, 16, 16)
