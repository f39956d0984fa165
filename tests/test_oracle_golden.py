"""The CPU FP64 oracle against the reference's own golden vectors.

Each test restates a reference test with the same data and tolerance:
  cpp/tests/kernels.cc:35-73            kernel values / corrections, abs 1e-13
  cpp/tests/operators.cc:64-101         G forward/adjoint 1e-5, S 1e-6
  cpp/tests/operators.cc:114-131        FFT round trip 1e-4
  cpp/tests/measurement_operator.cc     M31 forward, max-normalised, 1e-6
  cpp/tests/operators.cc:147-168        op norm ~ 1, determinism 1e-12
  cpp/tests/wproj_utils.cc:68-83        box Jw = 1 w-projection == plain G
"""
import numpy as np
import pytest

from conftest import golden, is_approx


@pytest.mark.parametrize("name", ["kb", "pswf", "gauss"])
def test_kernel_values(oracle_mod, name):
    g = golden("kernels")
    v = oracle_mod.kernel_values(name, 6, g["kernel_x"])
    assert np.abs(v - g["kernel_" + name]).max() < 1e-13


@pytest.mark.parametrize("name", ["kb", "pswf", "gauss"])
def test_kernel_corrections(oracle_mod, name):
    g = golden("kernels")
    v = oracle_mod.ft_kernel_values(name, 6, g["correction_x"])
    assert np.abs(v - g["correction_" + name]).max() < 1e-13


def test_bessel_i0_against_scipy(oracle_mod):
    sp = pytest.importorskip("scipy.special")
    x = np.linspace(0, 40, 2001)
    a = oracle_mod.bessel_i0(x)
    assert np.max(np.abs(a - sp.i0(x)) / sp.i0(x)) < 1e-13


def test_correction_S(oracle_mod):
    g = golden("operators")
    S = oracle_mod.correction("kb", 4, 4, 16, 16, 2.0)
    # Image<t_complex>::Map(expected_S, imsizey, imsizex) is column-major.
    expected = g["expected_S"].reshape(16, 16, order="F")
    assert is_approx(S, expected, 1e-6)


def test_gridding_matrix_forward_and_adjoint(oracle_mod):
    g = golden("operators")
    op = oracle_mod.Operator(g["u"], g["v"], None, None, 16, 16, 2.0, kernel="kb", Ju=4, Jv=4)
    assert op.nnz == 10 * 16
    d = op.G_forward(g["direct_input"])
    assert is_approx(d, g["expected_direct"], 1e-5)
    i = op.G_adjoint(g["indirect_input"])
    assert is_approx(i, g["expected_indirect"], 1e-5)


def test_fft_round_trip_and_numpy(oracle_mod):
    rng = np.random.default_rng(3)
    for shape in [(32, 32), (24, 40), (45, 16)]:
        a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        F = oracle_mod.fft2(a)
        assert np.allclose(F, np.fft.fft2(a) / np.sqrt(a.size), atol=1e-12)
        assert np.allclose(oracle_mod.fft2(F, inverse=True), a, atol=1e-12)


@pytest.mark.parametrize("name,J", [("kb", 4), ("pswf", 6), ("gauss", 6)])
def test_measurement_operator_m31(oracle_mod, name, J):
    m = golden("measurement_operator")
    x = m["m31"].astype(np.complex128)
    # the reference test swaps u and v at the call (measurement_operator.cc:36-39)
    op = oracle_mod.Operator(m["v"], m["u"], None, None, 256, 256, 2.0, power_iters=1,
                             power_tol=1e-9, kernel=name, Ju=J, Jv=J)
    y = op.forward(x)
    e = m[name + "_exact"]
    assert is_approx(y / np.abs(y).max(), e / np.abs(e).max(), 1e-6)


def _random_operator(oracle_mod, seed=0, M=1000, n=16, power_iters=10000, tol=1e-9):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1, 1, M)
    v = rng.uniform(-1, 1, M)
    w = rng.uniform(-1, 1, M)
    wt = rng.uniform(-1, 1, M) + 1j * rng.uniform(-1, 1, M)
    return oracle_mod.Operator(u, v, w, wt, n, n, 2.0, power_iters=power_iters, power_tol=tol,
                               kernel="kb", Ju=4, Jv=4)


def test_power_method_normalises(oracle_mod):
    op = _random_operator(oracle_mod)
    n2 = op.power_method(10000, 1e-9)  # on the unnormalised operator, sets the same norm
    rng = np.random.default_rng(5)
    x = rng.standard_normal(256) + 1j * rng.standard_normal(256)
    # normalised operator: ||Phi^H Phi|| ~ 1
    for _ in range(300):
        x = op.adjoint(op.forward(x))
        lam = np.linalg.norm(x)
        x /= lam
    assert abs(lam - 1.0) < 1e-6
    assert n2 > 0


def test_determinism(oracle_mod):
    op1 = _random_operator(oracle_mod, power_iters=50, tol=1e-6)
    op2 = _random_operator(oracle_mod, power_iters=50, tol=1e-6)
    rng = np.random.default_rng(7)
    a = rng.standard_normal(256) + 1j * rng.standard_normal(256)
    b = a.copy()
    for _ in range(100):
        a = op1.adjoint(op1.forward(a))
        b = op1.adjoint(op2.forward(b))
    assert is_approx(a, b, 1e-12)


def test_adjoint_dot_product(oracle_mod):
    op = _random_operator(oracle_mod, power_iters=20, tol=1e-6)
    rng = np.random.default_rng(9)
    x = rng.standard_normal(256) + 1j * rng.standard_normal(256)
    y = rng.standard_normal(op.M) + 1j * rng.standard_normal(op.M)
    lhs = np.vdot(y, op.forward(x))
    rhs = np.vdot(op.adjoint(y), x)
    assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(op.forward(x)) * np.linalg.norm(y)


def test_box_w_kernel_jw1_equals_plain_G(oracle_mod):
    rng = np.random.default_rng(11)
    M = 50
    u = rng.uniform(-30, 30, M)
    v = rng.uniform(-30, 30, M)
    w = rng.uniform(-50, 50, M)
    plain = oracle_mod.Operator(u, v, w, None, 32, 32, 2.0, kernel="kb", Ju=4, Jv=4)
    boxw = oracle_mod.Operator(u, v, w, None, 32, 32, 2.0, kernel="kb", Ju=4, Jv=4, w_term=True,
                               Jw=1, box_w=True)
    o1, i1, v1 = plain.G_matrix()
    o2, i2, v2 = boxw.G_matrix()
    assert plain.nnz == boxw.nnz
    assert np.array_equal(i1, i2)
    assert is_approx(v2, v1, 1e-12)


def test_lambda_to_pixels_round_trip(oracle_mod):
    # uvw units test (wproj_utils.cc:88-133): lambda = pixels * pixel_to_lambda
    for cell in (1.0, 3.0):
        u = np.ones(5)
        up, vp = oracle_mod.lambda_to_pixels(u, u, cell, cell, 256, 256)
        scale = 60.0 * 60.0 * 180.0 / cell / 256 / np.pi
        assert is_approx(u, up * scale, 1e-6)


def test_psf_convolve_normalised_norm_is_one(oracle_mod):
    """init_psf_convolve_2d's operator is normalised by its own power method,
    so a second power method gives norm 1 within power_tol
    (cpp/tests/operators.cc:201-214)."""
    rng = np.random.default_rng(0)
    n = 16
    u = rng.normal(0, 4, 200)
    v = rng.normal(0, 4, 200)
    op = oracle_mod.Operator(u, v, None, None, n, n, 2.0, kernel="kb", Ju=4, Jv=4)
    op.power_method(100, 1e-4)
    apply, norm = oracle_mod.psf_convolve(op, n, n, 100, 1e-4)
    assert norm > 0
    x = rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)
    x /= np.linalg.norm(x)
    for _ in range(300):
        x = apply(x)
        value = np.linalg.norm(x)
        x /= value
    assert abs(np.sqrt(value) - 1.0) < 1e-4
