"""Regenerate the golden fixtures in this folder from the reference's own data.

The reference keeps its golden vectors as text under ``data/expected`` and its
test image as ``data/images/M31.fits``.  This script parses them (the readers
of cpp/tests/data.in.h:14-48 and the FITS layout of cpp/purify/pfitsio.cc:186-205)
and stores the same numbers, unchanged, as compressed ``.npz`` fixtures so the
tests can run where the reference tree is not mounted.

Usage:  python tests/golden/make_golden.py REFERENCE_ROOT

REFERENCE_ROOT is the root of the reference checkout (the folder holding
``data/expected`` and ``data/images``); it has no default.
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_real(path):
    """Comma-separated reals (data.in.h:14-27)."""
    with open(path) as f:
        text = f.read()
    return np.array([float(t) for t in text.replace("\n", " ").split(",") if t.strip()],
                    dtype=np.float64)


def read_complex(path):
    """``(re,im)`` pairs (data.in.h:29-45)."""
    with open(path) as f:
        text = f.read()
    pairs = re.findall(r"\(\s*([^,()]+)\s*,\s*([^()]+)\s*\)", text)
    return np.array([complex(float(a), float(b)) for a, b in pairs], dtype=np.complex128)


def read_fits_image(path):
    """First image HDU of a BITPIX -32/-64 FITS file as a flat float array.

    NAXIS1 is the fastest axis of the file and becomes the fastest index of the
    flattened image vector (pfitsio.cc:186-205)."""
    with open(path, "rb") as f:
        raw = f.read()
    header = {}
    off = 0
    while True:
        block = raw[off:off + 2880]
        off += 2880
        done = False
        for k in range(36):
            card = block[80 * k:80 * (k + 1)].decode("ascii")
            key = card[:8].strip()
            if key == "END":
                done = True
                break
            if card[8:10] == "= ":
                header[key] = card[10:].split("/")[0].strip()
        if done:
            break
    bitpix = int(header["BITPIX"])
    naxis = [int(header["NAXIS%d" % (i + 1)]) for i in range(int(header["NAXIS"]))]
    n = int(np.prod(naxis))
    dtype = {-32: ">f4", -64: ">f8"}[bitpix]
    data = np.frombuffer(raw, dtype=dtype, count=n, offset=off)
    bscale = float(header.get("BSCALE", "1").replace("D", "E"))
    bzero = float(header.get("BZERO", "0").replace("D", "E"))
    assert bscale == 1.0 and bzero == 0.0
    return data.astype(data.dtype.newbyteorder("=")), naxis


def main(ref):
    exp = os.path.join(ref, "data", "expected")
    k = os.path.join(exp, "kernels")
    np.savez_compressed(
        os.path.join(HERE, "kernels.npz"),
        kernel_x=read_real(os.path.join(k, "kernel_x_data")),
        kernel_kb=read_real(os.path.join(k, "kernel_kb_data")),
        kernel_pswf=read_real(os.path.join(k, "kernel_pswf_data")),
        kernel_gauss=read_real(os.path.join(k, "kernel_gauss_data")),
        correction_x=read_real(os.path.join(k, "correction_x_data")),
        correction_kb=read_real(os.path.join(k, "correction_kb_data")),
        correction_pswf=read_real(os.path.join(k, "correction_pswf_data")),
        correction_gauss=read_real(os.path.join(k, "correction_gauss_data")),
    )
    o = os.path.join(exp, "operators")
    np.savez_compressed(
        os.path.join(HERE, "operators.npz"),
        u=read_real(os.path.join(o, "u_data")),
        v=read_real(os.path.join(o, "v_data")),
        direct_input=read_complex(os.path.join(o, "direct_input_data")),
        expected_direct=read_complex(os.path.join(o, "expected_direct_data")),
        indirect_input=read_complex(os.path.join(o, "indirect_input_data")),
        expected_indirect=read_complex(os.path.join(o, "expected_indirect_data")),
        expected_S=read_real(os.path.join(o, "expected_S_data")),
    )
    m = os.path.join(exp, "measurement_operator")
    img, naxis = read_fits_image(os.path.join(ref, "data", "images", "M31.fits"))
    np.savez_compressed(
        os.path.join(HERE, "measurement_operator.npz"),
        u=read_real(os.path.join(m, "u")),
        v=read_real(os.path.join(m, "v")),
        kb_exact=read_complex(os.path.join(m, "kb_exact_data")),
        pswf_exact=read_complex(os.path.join(m, "pswf_exact_data")),
        gauss_exact=read_complex(os.path.join(m, "gauss_exact_data")),
        m31=img,
        m31_naxis=np.array(naxis, dtype=np.int64),
    )
    # The first 400 rows of the reference's PADMM test coverage, unchanged,
    # as input for the .vis reader and the weighting tests.
    with open(os.path.join(exp, "padmm", "input_data.vis")) as f:
        head = [next(f) for _ in range(400)]
    with open(os.path.join(HERE, "padmm_input_head.vis"), "w") as f:
        f.writelines(head)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s REFERENCE_ROOT" % os.path.basename(sys.argv[0]))
    main(sys.argv[1])
