"""The C-ABI library loads, exports every symbol include/*.h declares, and
rejects bad requests before touching a GPU."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(purify_gb300_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_functions():
    assert len(declared_functions()) >= 20


def test_every_declared_symbol_is_exported(pg):
    lib = pg.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(pg.EXPORTS) == set(declared_functions())


def test_version_and_defaults(pg):
    lib = pg.load()
    assert b"sm_103a" in lib.purify_gb300_version()
    a = pg.CreateArgs()
    lib.purify_gb300_default_args(ctypes.byref(a))
    # defaults of measurementoperator::init_degrid_operator_2d (operators.h:373-380)
    assert a.oversample_ratio == 2.0 and a.power_iters == 100 and a.power_tol == 1e-4
    assert a.kernel == 0 and a.Ju == 4 and a.Jv == 4 and a.w_term == 0 and a.Jw == 6
    assert a.cellx == 1.0 and a.celly == 1.0


def _create(pg, **kw):
    u = np.zeros(4)
    args = dict(u=u, v=u, imsizey=16, imsizex=16, power_iters=0)
    args.update(kw)
    return pg.MeasurementOperator(**args)


@pytest.mark.parametrize("kw,status", [
    (dict(kernel="pswf", Ju=4, Jv=4), 1),   # kernels.cc:241-244
    (dict(kernel=17), 1),                   # kernels.cc:320-321
    (dict(Ju=4, Jv=6), 1),                  # KB: one axis outside its support (operators.h:322-324)
    (dict(kernel="kbmin", Ju=6, Jv=4), 1),
    (dict(kernel="gauss", Ju=4, Jv=6, w_term=True, w=np.zeros(4)), 2),
    (dict(Ju=33, Jv=33), 2),
    (dict(imsizex=0), 1),
    (dict(oversample_ratio=0.0), 1),
])
def test_invalid_requests_rejected_without_gpu(pg, kw, status):
    with pytest.raises(pg.PurifyError) as e:
        _create(pg, **kw)
    assert e.value.status == status


def test_mismatched_uv_lengths(pg):
    with pytest.raises(pg.PurifyError) as e:
        pg.MeasurementOperator(np.zeros(3), np.zeros(4), imsizey=8, imsizex=8, power_iters=0)
    assert e.value.status == 1


def test_null_pointers(pg):
    lib = pg.load()
    assert lib.purify_gb300_operator_create(None, None) == 1
    assert b"null" in lib.purify_gb300_last_error()
    assert lib.purify_gb300_forward(None, None, None, None) == 1


def test_correction_matches_golden(pg):
    from conftest import golden, is_approx
    g = golden("operators")
    S = pg.correction("kb", 4, 4, 16, 16, 2.0)
    assert is_approx(S, g["expected_S"].reshape(16, 16, order="F"), 1e-6)


def test_lambda_to_pixels(pg, oracle_mod):
    rng = np.random.default_rng(0)
    u = rng.normal(0, 1000, 100)
    v = rng.normal(0, 1000, 100)
    for cell in (0.0, 1.0, 2.5):
        a = pg.lambda_to_pixels(u, v, cell, cell, 512, 256)
        b = oracle_mod.lambda_to_pixels(u, v, cell, cell, 512, 256)
        assert np.allclose(a[0], b[0], rtol=1e-14) and np.allclose(a[1], b[1], rtol=1e-14)
