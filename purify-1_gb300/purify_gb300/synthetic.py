"""Seeded synthetic workloads for the measurement operator.

The reference measures on no public data set for this path; its benchmarks
draw random coverages (cpp/benchmarks/utilities.cc, utilities.cc:65-100).
These generators give reproducible stand-ins with the shapes of the
benchmark configurations (numpy PCG64, seeded):

* ``sky_image``: point sources (uniform positions, lognormal(0, 1) amplitudes)
  plus a centred Gaussian blob (sigma 8 px, peak 1).
* ``gaussian_core_uv``: u, v ~ N(0, sigma^2) in grid pixels, redrawn until
  inside [-N/2, N/2).
* ``mixed_uv``: a fraction from the Gaussian core, the rest uniform over the
  grid.
"""
import numpy as np


def sky_image(imsizey, imsizex, n_sources=50, blob_sigma=8.0, seed=0):
    rng = np.random.default_rng(seed)
    img = np.zeros((imsizey, imsizex), dtype=np.float64)
    ys = rng.integers(0, imsizey, n_sources)
    xs = rng.integers(0, imsizex, n_sources)
    amp = rng.lognormal(0.0, 1.0, n_sources)
    np.add.at(img, (ys, xs), amp)
    yy, xx = np.mgrid[0:imsizey, 0:imsizex]
    cy, cx = (imsizey - 1) / 2.0, (imsizex - 1) / 2.0
    img += np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * blob_sigma ** 2))
    return img.astype(np.complex128).ravel()


def _clipped_normal(rng, n, sigma, half):
    out = rng.normal(0.0, sigma, n)
    bad = (out < -half) | (out >= half)
    while bad.any():
        out[bad] = rng.normal(0.0, sigma, int(bad.sum()))
        bad = (out < -half) | (out >= half)
    return out


def gaussian_core_uv(M, ftsizeu, ftsizev, sigma_frac, seed=0, scale=1.0):
    """sigma = sigma_frac * ftsize / 2 per axis (pixels), times `scale`."""
    rng = np.random.default_rng(seed)
    u = _clipped_normal(rng, M, sigma_frac * ftsizeu / 2.0 * scale, ftsizeu / 2.0)
    v = _clipped_normal(rng, M, sigma_frac * ftsizev / 2.0 * scale, ftsizev / 2.0)
    return u, v


def mixed_uv(M, ftsizeu, ftsizev, core_frac=0.7, sigma_frac=0.15, seed=0):
    """core_frac of the points with sigma = sigma_frac * N (pixels, N the grid
    size), the rest uniform over [-N/2, N/2); shuffled together."""
    rng = np.random.default_rng(seed)
    mc = int(round(M * core_frac))
    u = np.empty(M)
    v = np.empty(M)
    u[:mc] = _clipped_normal(rng, mc, sigma_frac * ftsizeu, ftsizeu / 2.0)
    v[:mc] = _clipped_normal(rng, mc, sigma_frac * ftsizev, ftsizev / 2.0)
    u[mc:] = rng.uniform(-ftsizeu / 2.0, ftsizeu / 2.0, M - mc)
    v[mc:] = rng.uniform(-ftsizev / 2.0, ftsizev / 2.0, M - mc)
    p = rng.permutation(M)
    return u[p], v[p]


def random_vis(M, seed=1):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex128)


def config_small(seed=0):
    """256^2 image, 512^2 grid, 1e5 visibilities, u,v ~ N(0, (0.25 * 512 / 2)^2), KB J=4."""
    u, v = gaussian_core_uv(100_000, 512, 512, 0.25, seed=seed)
    return dict(u=u, v=v, imsizey=256, imsizex=256, kernel="kb", Ju=4, Jv=4,
                x=sky_image(256, 256, seed=seed))


def config_large(M=10_000_000, seed=0):
    """1024^2 image, 2048^2 grid, KB J=6, 70% core (sigma 0.15 N) + 30% uniform."""
    u, v = mixed_uv(M, 2048, 2048, 0.7, 0.15, seed=seed)
    return dict(u=u, v=v, imsizey=1024, imsizex=1024, kernel="kb", Ju=6, Jv=6,
                x=sky_image(1024, 1024, seed=seed))


def wproj_supports(w, w_max, J=4, s_min=4, s_max=24):
    """Per-row w-supports for the w-projection workload: the total support
    S = Jw + J - 1 grows affinely with |w - mean(w)| from s_min at w = 0 to
    s_max at |w| = w_max; returns Jw per row."""
    wc = np.abs(np.asarray(w) - np.mean(w))
    S = np.clip(np.rint(s_min + (s_max - s_min) * wc / w_max), s_min, s_max).astype(np.int32)
    return S - (J - 1)


def config_wproj(M=20_000_000, imsize=2048, cell=1.0, seed=0):
    """2048^2 image, 4096^2 grid, 70% core + 30% uniform uv, w ~ U(-w_max,
    w_max) with w_max = 12 grid pixels in wavelengths (so the validity region
    of the small-angle w-kernel spans about 24 taps at |w| = w_max), KB J=4,
    per-row support 4..24 taps per axis."""
    N = 2 * imsize
    u, v = mixed_uv(M, N, N, 0.7, 0.15, seed=seed)
    du = 60.0 * 60.0 * 180.0 / cell / N / np.pi
    w_max = 12.0 * du
    w = np.random.default_rng(seed + 17).uniform(-w_max, w_max, M)
    return dict(u=u, v=v, w=w, jw_rows=wproj_supports(w, w_max), imsizey=imsize, imsizex=imsize,
                cellx=cell, celly=cell, kernel="kb", Ju=4, Jv=4, w_max=w_max,
                x=sky_image(imsize, imsize, seed=seed))


def config_batch(nch=64, seed=0, m_lo=1e4, m_hi=2e6, sizes=(256, 512, 1024)):
    """nch frequency channels: image size drawn from `sizes`, visibility count
    log-uniform in [m_lo, m_hi], coverage 70% Gaussian core with sigma =
    0.15 N (1 + 0.01 k) (channel frequency) + 30% uniform, KB J=4."""
    rng = np.random.default_rng(seed)
    sz = rng.choice(np.asarray(sizes), nch)
    Ms = np.exp(rng.uniform(np.log(m_lo), np.log(m_hi), nch)).astype(np.int64)
    chans = []
    for k in range(nch):
        n = int(sz[k])
        u, v = mixed_uv(int(Ms[k]), 2 * n, 2 * n, 0.7, 0.15 * (1 + 0.01 * k), seed=seed + 1000 + k)
        chans.append(dict(u=u, v=v, imsizey=n, imsizex=n, x=sky_image(n, n, seed=seed + k)))
    return chans


def config_serve_pool(n=16, seed=0, m_lo=1e4, m_hi=5e6, sizes=(256, 512, 1024)):
    """n resident coverages for the request server: image size drawn from
    `sizes`, visibility count log-uniform in [m_lo, m_hi], 70% Gaussian core
    (sigma = 0.15 N) + 30% uniform, KB J=4."""
    rng = np.random.default_rng(seed)
    sz = rng.choice(np.asarray(sizes), n)
    Ms = np.exp(rng.uniform(np.log(m_lo), np.log(m_hi), n)).astype(np.int64)
    out = []
    for k in range(n):
        m = int(sz[k])
        u, v = mixed_uv(int(Ms[k]), 2 * m, 2 * m, 0.7, 0.15, seed=seed + 2000 + k)
        out.append(dict(u=u, v=v, imsizey=m, imsizex=m))
    return out


def request_stream(n, rate, n_coverages, seed=0, mix=(0.70, 0.25, 0.05)):
    """n requests of a Poisson stream at `rate` per second: arrival times,
    kinds (forward_adjoint / adjoint / norm with probabilities `mix`) and
    coverages (uniform over the pool)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    kinds = rng.choice(np.array(["forward_adjoint", "adjoint", "norm"]), n, p=np.asarray(mix))
    cov = rng.integers(0, n_coverages, n)
    return t, kinds, cov
