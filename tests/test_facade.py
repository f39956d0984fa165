"""The C++ face (include/purify_gb300.hpp): compiles against the C ABI
without sopt / Eigen (CPU), and on a GPU gives the oracle's Phi / Phi^H."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_l2

SRC = os.path.join(ROOT, "tests", "cpp", "facade_test.cpp")


def build_facade(tmp_path, pg):
    lib = pg.build()
    exe = os.path.join(str(tmp_path), "facade_test")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
                    "-L", libdir, "-Wl,-rpath," + libdir, "-lpurify_gb300"], check=True)
    return exe


def test_facade_compiles_and_links(tmp_path, pg):
    assert os.path.exists(build_facade(tmp_path, pg))


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
