"""A second, independent restatement of the reference's w-projection rows,
written with numpy / scipy.signal and checked against the oracle's CSR rows.

The oracle (C++) and the device factor storage are both readings of the same
reference code; this file reads it a third time, straight from the formulas,
so that an error shared by the first two readings does not go unnoticed:

* projection_kernels.cc:59-85 — the separable taps kernelu(du - j - 1) on both
  axes (the v axis also calls kernelu), du = u - floor(u - J/2), and the
  Jw x Jw w-kernel samples kernelw(dwu - ju - 1, dwv - jv - 1, w);
* projection_kernels.cc:16-47 — the small-angle w-kernel
  exp(-i pi (U^2 + V^2) / w) / (w i) at U = u du_l, V = v dv_l with
  du_l = 3600 * 180 / (cell * floor(os * N) * pi), and 1 outside the
  rectangle |U / w| < 1, |V / w| < 1;
* convolution.h:54-82 — linear_convol_2d: a 1-D "linear_convol_1d" over the
  columns with the v taps, then over the rows with the u taps, on zero-padded
  inputs.  linear_convol_1d(f, g)(j) = sum_k f(k) g(Jg - 1 - j + k), which is
  numpy.convolve(f, g[::-1]); the 2-D form is therefore
  scipy.signal.convolve2d(g[::-1, ::-1], outer(kv, ku));
* operators.cc:73-96 — row placement kw = floor(u - (Jw + J - 1) / 2), taps at
  kw + 1 .. kw + S (mod N), value exp(-2 pi i ((kwu + ju) / 2 + (kwv + jv) / 2))
  * K(jv - 1, ju - 1) * weight;
* operators.h:323 — the rows see w - mean(w).
"""
import numpy as np
import pytest
import scipy.signal
import scipy.special


def kb(x, J):
    """kernels::kaiser_bessel (kernels.cc:7-22)."""
    alpha = 2.34 * J
    a = 2.0 * x / J
    return scipy.special.i0(alpha * np.sqrt(1.0 - a * a)) / scipy.special.i0(alpha)


def w_sample(U, V, w, du_l, dv_l):
    """w_projection_kernel_approx (projection_kernels.cc:31-47)."""
    if abs(U * du_l / w) < 1 and abs(V * dv_l / w) < 1:
        Ul, Vl = U * du_l, V * dv_l
        return np.exp(-1j * np.pi * (Ul * Ul + Vl * Vl) / w) / w / 1j
    return 1.0 + 0j


def reference_row(u, v, w, weight, J, Jw, n, os, cell):
    """{grid index: value} of one w-projection row of G."""
    N = int(np.floor(os * n))
    du_l = dv_l = 60.0 * 60.0 * 180.0 / cell / N / np.pi
    du = u - np.floor(u - J * 0.5)
    dv = v - np.floor(v - J * 0.5)
    ku = np.array([kb(du - j - 1, J) for j in range(J)])
    kv = np.array([kb(dv - j - 1, J) for j in range(J)])  # kernelu on the v axis too
    dwu = u - np.floor(u - Jw * 0.5)
    dwv = v - np.floor(v - Jw * 0.5)
    g = np.array([[w_sample(dwu - iu - 1, dwv - jv - 1, w, du_l, dv_l) for iu in range(Jw)]
                  for jv in range(Jw)])
    K = scipy.signal.convolve2d(g[::-1, ::-1], np.outer(kv, ku))
    S = Jw + J - 1
    assert K.shape == (S, S)
    kwu = np.floor(u - S * 0.5)
    kwv = np.floor(v - S * 0.5)
    row = {}
    for ju in range(1, S + 1):
        for jv in range(1, S + 1):
            q = int(np.mod(kwu + ju, N))
            p = int(np.mod(kwv + jv, N))
            phase = np.exp(-2j * np.pi * ((kwu + ju) * 0.5 + (kwv + jv) * 0.5))
            row[p * N + q] = row.get(p * N + q, 0) + phase * K[jv - 1, ju - 1] * weight
    return row


@pytest.mark.parametrize("Jw,cell", [(6, 1.0), (13, 1.0), (9, 2.5)])
def test_oracle_w_rows_match_independent_restatement(oracle_mod, Jw, cell):
    n, M, os, J = 64, 400, 2.0, 4
    N = int(os * n)
    rng = np.random.default_rng(Jw)
    u = rng.normal(0, N / 8, M)
    v = rng.normal(0, N / 8, M)
    du_l = 60.0 * 60.0 * 180.0 / cell / N / np.pi
    w = rng.uniform(-12 * du_l, 12 * du_l, M)
    wt = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    op = oracle_mod.Operator(u, v, w, wt, n, n, os, kernel="kb", Ju=J, Jv=J, w_term=True, Jw=Jw,
                             cellx=cell, celly=cell)
    off, idx, val = op.G_matrix()
    wc = w - w.mean()
    worst = 0.0
    for m in range(0, M, 7):  # about 60 rows
        ref = reference_row(u[m], v[m], wc[m], wt[m], J, Jw, n, os, cell)
        got = {}
        for k in range(off[m], off[m + 1]):
            got[int(idx[k])] = got.get(int(idx[k]), 0) + val[k]
        assert set(got) == set(ref)
        scale = max(abs(x) for x in ref.values())
        err = max(abs(got[k] - ref[k]) for k in ref) / scale
        worst = max(worst, err)
    # FP64 rounding at the row's scale: the median row agrees to 7e-16; a row
    # whose chirp convolution sums cancel by about three digits reaches 2e-12
    assert worst < 1e-11, worst
