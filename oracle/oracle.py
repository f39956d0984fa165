"""ctypes wrapper of the CPU FP64 oracle (``purify_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: the parity checker for the GB300 measurement
operator.  tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it; the product library never imports it.

The oracle restates the reference operator in complex<double> with the
reference's own structure (explicit CSR G and G^H, row-parallel SpMV, unitary
2-D FFT); ``purify_oracle.cpp`` cites the reference file:line of each piece.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

KERNELS = {"kb": 0, "gauss": 1, "box": 2, "pswf": 3, "kbmin": 4, "gauss_alt": 5}

_lib = None


def build():
    """Compile the oracle with its Makefile (g++ -fopenmp)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        d, i64, i32, vp = ctypes.c_double, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
        P = ctypes.POINTER
        L.or_last_error.restype = ctypes.c_char_p
        L.or_create.restype = vp
        L.or_create.argtypes = [vp, vp, vp, vp, i64, i32, i32, d, i32, i32, i32, i32, i32, d, d,
                                vp, i32]
        L.or_destroy.argtypes = [vp]
        L.or_nnz.restype = i64
        L.or_nnz.argtypes = [vp]
        L.or_shape.argtypes = [vp, vp]
        L.or_get_G.argtypes = [vp, vp, vp, vp]
        for f in (L.or_G_forward, L.or_G_adjoint, L.or_forward, L.or_adjoint):
            f.argtypes = [vp, vp, vp]
        L.or_set_norm.argtypes = [vp, d]
        L.or_get_norm.restype = d
        L.or_get_norm.argtypes = [vp]
        L.or_power_method.argtypes = [vp, i32, d, vp, P(d)]
        L.or_kernel_values.argtypes = [i32, i32, d, vp, i64, vp]
        L.or_ft_kernel_values.argtypes = [i32, i32, d, vp, i64, vp]
        L.or_bessel_i0.argtypes = [vp, i64, vp]
        L.or_correction.argtypes = [i32, i32, i32, i32, i32, d, vp]
        L.or_fft2.argtypes = [i32, i32, vp, vp, i32]
        L.or_set_threads.argtypes = [i32]
        L.or_get_threads.restype = i32
        L.or_lambda_to_pixels.argtypes = [vp, vp, i64, d, d, i32, i32, vp, vp]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _check(rc):
    if rc != 0:
        raise RuntimeError(lib().or_last_error().decode())


def set_threads(n):
    lib().or_set_threads(int(n))


def get_threads():
    return lib().or_get_threads()


def kernel_values(kernel, J, x, oversample=2.0):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    _check(lib().or_kernel_values(KERNELS[kernel], J, oversample, _ptr(x), x.size, _ptr(out)))
    return out


def ft_kernel_values(kernel, J, x, oversample=2.0):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    _check(lib().or_ft_kernel_values(KERNELS[kernel], J, oversample, _ptr(x), x.size, _ptr(out)))
    return out


def bessel_i0(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    _check(lib().or_bessel_i0(_ptr(x), x.size, _ptr(out)))
    return out


def correction(kernel, Ju, Jv, imsizey, imsizex, oversample=2.0):
    """S(j, i) as an (imsizey, imsizex) complex array."""
    out = np.empty(imsizey * imsizex, dtype=np.complex128)
    _check(lib().or_correction(KERNELS[kernel], Ju, Jv, imsizey, imsizex, oversample, _ptr(out)))
    return out.reshape(imsizey, imsizex)


def fft2(a, inverse=False):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    out = np.empty_like(a)
    _check(lib().or_fft2(a.shape[0], a.shape[1], _ptr(a), _ptr(out), 1 if inverse else 0))
    return out


def lambda_to_pixels(u, v, cellx, celly, ftsizeu, ftsizev):
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    uo, vo = np.empty_like(u), np.empty_like(v)
    lib().or_lambda_to_pixels(_ptr(u), _ptr(v), u.size, cellx, celly, ftsizeu, ftsizev, _ptr(uo),
                              _ptr(vo))
    return uo, vo


class Operator:
    """FP64 measurement operator Phi = G F Z S / norm (oracle).

    Mirrors ``measurementoperator::init_degrid_operator_2d`` with u, v, w in
    pixels (cpp/purify/operators.h:372-396).  ``power_iters`` > 0 runs the power
    method and normalises; ``jw_rows`` gives per-row w-supports and ``box_w``
    selects the box w-kernel (test identities only)."""

    def __init__(self, u, v, w, weights, imsizey, imsizex, oversample_ratio=2.0,
                 power_iters=0, power_tol=1e-4, kernel="kb", Ju=4, Jv=4, w_term=False, Jw=6,
                 cellx=1.0, celly=1.0, jw_rows=None, box_w=False):
        self.u = np.ascontiguousarray(u, dtype=np.float64)
        self.v = np.ascontiguousarray(v, dtype=np.float64)
        M = self.u.size
        self.w = np.ascontiguousarray(w if w is not None else np.zeros(M), dtype=np.float64)
        self.weights = np.ascontiguousarray(
            weights if weights is not None else np.ones(M), dtype=np.complex128)
        jw = None if jw_rows is None else np.ascontiguousarray(jw_rows, dtype=np.int32)
        self._jw = jw
        self.h = lib().or_create(_ptr(self.u), _ptr(self.v), _ptr(self.w), _ptr(self.weights), M,
                                 imsizey, imsizex, oversample_ratio, KERNELS[kernel], Ju, Jv,
                                 1 if w_term else 0, Jw, cellx, celly, _ptr(jw),
                                 1 if box_w else 0)
        if not self.h:
            raise RuntimeError(lib().or_last_error().decode())
        shape = np.zeros(6, dtype=np.int64)
        lib().or_shape(self.h, _ptr(shape))
        self.M, self.imsizey, self.imsizex, self.ftsizev, self.ftsizeu, self.nnz = map(int, shape)
        self.norm = 1.0
        if power_iters > 0:
            self.power_method(power_iters, power_tol)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().or_destroy(h)
            self.h = None

    def G_matrix(self):
        """(offsets, index, values) of the CSR G."""
        off = np.empty(self.M + 1, dtype=np.int64)
        idx = np.empty(self.nnz, dtype=np.int32)
        val = np.empty(self.nnz, dtype=np.complex128)
        lib().or_get_G(self.h, _ptr(off), _ptr(idx), _ptr(val))
        return off, idx, val

    def G_forward(self, grid):
        grid = np.ascontiguousarray(grid, dtype=np.complex128).ravel()
        out = np.empty(self.M, dtype=np.complex128)
        lib().or_G_forward(self.h, _ptr(grid), _ptr(out))
        return out

    def G_adjoint(self, vis):
        vis = np.ascontiguousarray(vis, dtype=np.complex128).ravel()
        out = np.empty(self.ftsizeu * self.ftsizev, dtype=np.complex128)
        lib().or_G_adjoint(self.h, _ptr(vis), _ptr(out))
        return out

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128).ravel()
        out = np.empty(self.M, dtype=np.complex128)
        lib().or_forward(self.h, _ptr(x), _ptr(out))
        return out

    def adjoint(self, y):
        y = np.ascontiguousarray(y, dtype=np.complex128).ravel()
        out = np.empty(self.imsizey * self.imsizex, dtype=np.complex128)
        lib().or_adjoint(self.h, _ptr(y), _ptr(out))
        return out

    def set_norm(self, norm):
        self.norm = float(norm)
        lib().or_set_norm(self.h, self.norm)

    def power_method(self, iters, tol, x0=None):
        x0 = None if x0 is None else np.ascontiguousarray(x0, dtype=np.complex128).ravel()
        out = ctypes.c_double()
        _check(lib().or_power_method(self.h, int(iters), float(tol), _ptr(x0), ctypes.byref(out)))
        self.norm = out.value
        return self.norm


def psf_convolve(op, imsizey, imsizex, power_iters=100, power_tol=1e-4):
    """operators::init_psf_convolve_2d (cpp/purify/compact_operators.h:279-307)
    on an oracle operator: psf = Phi^H Phi delta with delta at sub2ind(floor(Ny/2)
    - 1, floor(Nx/2) - 1) (utilities.cc:321-333, row * cols + col); A x =
    F^-1(F psf . F x) with the unitary Ny x Nx FFT of init_FFT_2d
    (operators.h:206-261; no padding, circular); the power method on {A, id}
    (the rule of Operator.power_method, from a fixed pseudo-random image)
    gives ||A||, and the operator is A / ||A||^2.  Returns (apply, norm)."""
    N = imsizey * imsizex
    delta = np.zeros(N, dtype=np.complex128)
    delta[(imsizey // 2 - 1) * imsizex + (imsizex // 2 - 1)] = 1.0
    psf = op.adjoint(op.forward(delta))
    # fft2 is the oracle's unitary transform (each direction / sqrt(N))
    ft = fft2(psf.reshape(imsizey, imsizex)).ravel()

    def raw(x):
        fx = fft2(np.asarray(x, dtype=np.complex128).reshape(imsizey, imsizex)).ravel()
        return fft2((ft * fx).reshape(imsizey, imsizex), inverse=True).ravel()

    norm = 1.0
    if power_iters > 0:
        # start: x_k = h(k) / 2^32 - 1/2, h(k) = 2654435761 k mod 2^32 (Knuth's
        # multiplicative hash), normalised -- the all-ones image is the
        # zero-frequency eigenvector of a circular convolution, so the
        # reference starts from a random image instead
        k = np.arange(N, dtype=np.uint64)
        x = ((k * np.uint64(2654435761)) % np.uint64(2 ** 32)).astype(np.float64) / 2.0 ** 32 - 0.5
        x = (x / np.linalg.norm(x)).astype(np.complex128)
        old = 0.0
        for _ in range(power_iters):
            x = raw(x)
            value = float(np.sqrt(np.sum(np.abs(x) ** 2)))
            if not value > 0:
                raise RuntimeError("Operator norm is not greater than zero.")
            x = x / value
            if power_tol * power_tol > abs(old - value) / old if old else False:
                old = value
                break
            old = value
        norm = float(np.sqrt(old))
    return (lambda x: raw(x) / norm ** 2), norm


def read_visibility(path, w_term=False):
    """utilities::read_visibility (cpp/purify/utilities.cc:140-188) restated:
    rows of u v [w] re im sigma; v negated (utilities.cc:178), weight 1 / sigma."""
    with open(path) as f:
        rows = sum(1 for _ in f)
    with open(path) as f:
        toks = f.read().split()
    per = 6 if w_term else 5
    vals = np.array([float(t) for t in toks[:rows * per]], dtype=np.float64).reshape(rows, per)
    u, v = vals[:, 0], -vals[:, 1]
    w = vals[:, 2] if w_term else np.zeros(rows)
    k = 3 if w_term else 2
    vis = np.empty(rows, dtype=np.complex128)
    vis.real, vis.imag = vals[:, k], vals[:, k + 1]
    weights = np.zeros(rows, dtype=np.complex128)
    weights.real = 1.0 / vals[:, k + 2]
    return {"u": u.copy(), "v": v.copy(), "w": w.copy(), "vis": vis, "weights": weights}


def init_weights(u, v, weights, oversample_factor, weighting, R, ftsizeu, ftsizev):
    """utilities::init_weights (cpp/purify/utilities.cc:569-608) restated with
    sequential loops; utilities::mod is fmod wrapped to [0, y)."""
    weights = np.asarray(weights, dtype=np.complex128)
    if weighting == "none":
        return np.ones_like(weights)
    if weighting in ("natural", "whiten"):
        return weights.copy()
    if weighting not in ("uniform", "robust"):
        raise RuntimeError("Wrong weighting type, " + weighting + " not recognised.")
    scale = 1.0 / oversample_factor
    q = np.mod(np.floor(np.asarray(u) * scale), ftsizeu).astype(np.int64)
    p = np.mod(np.floor(np.asarray(v) * scale), ftsizev).astype(np.int64)
    grid = np.zeros((ftsizev, ftsizeu), dtype=np.complex128)
    for a, b in zip(p, q):
        grid[a, b] += 1
    sum_weights = np.sum(weights * weights)
    sum_grid2 = np.sum(grid * grid)
    robust_scale = sum_weights / sum_grid2 * 25.0 * 10.0 ** (-2 * R)
    g = np.sqrt(grid)
    if weighting == "uniform":
        return weights / g[p, q]
    return weights / np.sqrt(1.0 + robust_scale * g[p, q] * g[p, q])
