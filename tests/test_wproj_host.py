"""w-projection rows on the CPU: the factors the device stores (only the
nonzero terms of the rank-3 split: rank 1 where the validity rectangle covers
all samples or none, up to 3 otherwise) rebuild the reference's row values
(operators.cc:49-99 with projection_kernels.cc:16-85), compared with the
oracle's explicit CSR rows."""
import numpy as np
import pytest

CASES = [
    # u, v (pixels), w (wavelengths, after mean removal), Jw, J, cell (arcsec)
    (0.3, -0.7, 0.0, 6, 4, 1.0),       # w = 0: the sample is 1 everywhere
    (1.25, 2.5, 400.0, 6, 4, 1.0),     # partly valid rectangle
    (-3.6, 4.1, -900.0, 9, 4, 1.0),
    (5.5, -2.2, 50000.0, 12, 4, 1.0),  # fully valid
    (0.5, 0.5, 123.0, 1, 4, 3.0),      # Jw = 1
    (2.2, 1.1, 1500.0, 7, 6, 1.0),     # odd support with J = 6
]


@pytest.mark.parametrize("u,v,w,Jw,J,cell", CASES)
def test_wrow_factors_rebuild_reference_rows(pg, oracle_mod, u, v, w, Jw, J, cell):
    n = 64
    # an even shift keeps the taps and the phase and keeps the footprint off
    # the grid edge, so the CSR column order is row-major (v, u)
    u, v = u + 40, v + 40
    K = pg.wrow_taps(u, v, w, Jw, J, "kb", 2.0, n, n, cell, cell)
    uu, vv, ww = np.array([u, u]), np.array([v, v]), np.array([w, -w])
    op = oracle_mod.Operator(uu, vv, ww, None, n, n, 2.0, kernel="kb", Ju=J, Jv=J, w_term=True,
                             Jw=Jw, cellx=cell, celly=cell)
    off, idx, val = op.G_matrix()
    S = Jw + J - 1
    row = val[off[0]:off[1]]
    # the footprint does not wrap here, so column order is row-major (v, u)
    assert row.size == S * S
    # to FP64 rounding at the row's scale.  The factor terms have disjoint
    # supports in the sample matrix, so none cancels another (a split with
    # 1 1^T - chi chi^T terms loses ~5 digits at w = 5e4); what remains is the
    # reference's own convolution of an oscillating chirp, whose sums cancel
    # up to ~3 digits and amplify rounding accordingly.
    assert np.abs(K.ravel() - row).max() <= 1e-11 * np.abs(row).max()
