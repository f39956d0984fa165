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
