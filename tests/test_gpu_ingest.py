"""Uniform and robust visibility weighting on the GPU against the oracle's
restatement of utilities::init_weights (utilities.cc:569-608).  The counts
are exact (integer atomics); the sums are FP64 in a fixed order, so the
weights agree with the sequential restatement to rounding: relative 1e-13."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from purify_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,R", [("uniform", 0.0), ("robust", 0.0), ("robust", 1.5),
                                    ("robust", -1.0)])
def test_weights_on_reference_coverage(pg, oracle_mod, cuda, kind, R):
    d = pg.read_visibility(os.path.join(GOLDEN, "padmm_input_head.vis"))
    # the PADMM coverage in grid pixels of a 128^2 grid (lambda -> pixels as the reference does)
    u, v = pg.lambda_to_pixels(d["u"], d["v"], 0.0, 0.0, 128, 128)
    got = pg.init_weights(u, v, d["weights"], 2.0, kind, R, 128, 128)
    ref = oracle_mod.init_weights(u, v, d["weights"], 2.0, kind, R, 128, 128)
    assert np.max(np.abs(got - ref) / np.abs(ref)) < 1e-13


@pytest.mark.parametrize("kind", ["uniform", "robust"])
def test_weights_large_coverage(pg, oracle_mod, cuda, kind):
    u, v = synthetic.mixed_uv(200_000, 512, 512, 0.7, 0.15, seed=11)
    rng = np.random.default_rng(3)
    w = rng.uniform(0.5, 2.0, u.size) + 0.1j * rng.standard_normal(u.size)
    got = pg.init_weights(u, v, w, 2.0, kind, 0.5, 512, 512)
    ref = oracle_mod.init_weights(u, v, w, 2.0, kind, 0.5, 512, 512)
    assert np.max(np.abs(got - ref) / np.abs(ref)) < 1e-13
