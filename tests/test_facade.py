"""The C++ face (include/purify_gb300.hpp): compiles against the C ABI
without sopt / Eigen (CPU), throws std::runtime_error on the reference's
size errors (CPU), and on a GPU gives the oracle's Phi / Phi^H, through the
raw overload and through the vis_params overload in all three units."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_l2

SRC = os.path.join(ROOT, "tests", "cpp", "facade_test.cpp")
ERRORS_SRC = os.path.join(ROOT, "tests", "cpp", "facade_errors.cpp")


def build_facade(tmp_path, pg, src=SRC, name="facade_test"):
    lib = pg.build()
    exe = os.path.join(str(tmp_path), name)
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), src, "-o", exe,
                    "-L", libdir, "-Wl,-rpath," + libdir, "-lpurify_gb300"], check=True)
    return exe


def test_facade_compiles_and_links(tmp_path, pg):
    assert os.path.exists(build_facade(tmp_path, pg))


def test_facade_size_errors_throw(tmp_path, pg):
    """u / v, weights and (with w_term) w sizes that differ from M, and an
    unknown unit, are std::runtime_error before any device work."""
    exe = build_facade(tmp_path, pg, ERRORS_SRC, "facade_errors")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count(" threw") == 6, r.stdout


def test_units_pipeline(pg, oracle_mod):
    """vis_params units (operators.h:405-410): wavelengths as set_cell_size +
    uv_scale, radians as uv_scale, pixels unchanged."""
    rng = np.random.default_rng(0)
    u = rng.normal(0, 300, 1000)
    v = rng.normal(0, 300, 1000)
    a = pg.uv_to_pixels(u, v, "lambda", 0.5, 0.7, 512, 256)
    b = oracle_mod.lambda_to_pixels(u, v, 0.5, 0.7, 512, 256)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    ur, vr = u * 1e-3, v * 1e-3
    a = pg.uv_to_pixels(ur, vr, "radians", 0.0, 0.0, 512, 256)
    assert np.array_equal(a[0], ur / (2 * np.pi) * 512)
    assert np.array_equal(a[1], vr / (2 * np.pi) * 256)
    a = pg.uv_to_pixels(u, v, "pixels", 0.0, 0.0, 512, 256)
    assert np.array_equal(a[0], u) and np.array_equal(a[1], v)
    with pytest.raises(pg.PurifyError):
        pg.uv_to_pixels(u, v, 5, 0.0, 0.0, 512, 256)


@pytest.mark.gpu
def test_facade_matches_oracle(tmp_path, pg, oracle_mod, cuda):
    exe = build_facade(tmp_path, pg)
    rng = np.random.default_rng(3)
    M, n = 3000, 48
    u = rng.normal(0, 20, M)
    v = rng.normal(0, 20, M)
    x = rng.standard_normal(n * n) + 1j * rng.standard_normal(n * n)
    y = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    inp = os.path.join(str(tmp_path), "in.bin")
    out = os.path.join(str(tmp_path), "out.bin")
    with open(inp, "wb") as f:
        np.array([M, n], dtype=np.int64).tofile(f)
        u.tofile(f)
        v.tofile(f)
        x.astype(np.complex128).tofile(f)
        y.astype(np.complex128).tofile(f)
    r = subprocess.run([exe, inp, out], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    data = np.fromfile(out, dtype=np.float64)
    fx = data[1:1 + 2 * M].view(np.complex128)
    ay = data[1 + 2 * M:].view(np.complex128)
    ref = oracle_mod.Operator(u, v, None, None, n, n, 2.0, power_iters=50, power_tol=1e-4,
                              kernel="kb", Ju=4, Jv=4)
    assert rel_l2(fx, ref.forward(x)) < 1e-10
    assert rel_l2(ay, ref.adjoint(y)) < 1e-10
