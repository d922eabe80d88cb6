"""Seeded synthetic inputs for the cell-centred MLMG workloads.

The workloads are defined on the unit cube [0,1]^3 with cell-centred data:

* ``gaussian_rhs`` -- a right-hand side made of a sum of Gaussian blobs with
  centres uniform in the domain, widths uniform in [0.02, 0.1] and amplitudes
  drawn from N(0, 1).
* ``lognormal_bcoef`` -- face b-coefficients exp(contrast * g), where g is a
  Gaussian random field (white noise convolved with a Gaussian kernel of
  ``sigma_cells`` cells, normalised to zero mean and unit variance).  The
  field is generated on the domain grown by one cell, and each face value is
  the mean of its two adjacent cell values, so every face of the domain
  (boundary faces included) has a well-defined coefficient.
* ``smooth_field`` -- a smooth random target field made by the same generator.

All generators use numpy's PCG64 with an explicit seed so that the GPU solver,
the C oracle and the reference driver read identical bytes.  Arrays are
float64, C-ordered as (nz, ny, nx) -- x fastest, the same order as an AMReX
FArrayBox.
"""
from __future__ import annotations

import numpy as np


def cell_centres(n):
    nx, ny, nz = n
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    z = (np.arange(nz) + 0.5) / nz
    return x, y, z


def gaussian_rhs(n, seed, nblobs=16, wmin=0.02, wmax=0.1):
    """Sum of ``nblobs`` Gaussian blobs sampled at cell centres."""
    n = _as3(n)
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(0.0, 1.0, size=(nblobs, 3))
    w = rng.uniform(wmin, wmax, size=nblobs)
    amp = rng.standard_normal(nblobs)
    x, y, z = cell_centres(n)
    out = np.zeros((n[2], n[1], n[0]), dtype=np.float64)
    for k in range(nblobs):
        gx = np.exp(-((x - c[k, 0]) ** 2) / (2 * w[k] ** 2))
        gy = np.exp(-((y - c[k, 1]) ** 2) / (2 * w[k] ** 2))
        gz = np.exp(-((z - c[k, 2]) ** 2) / (2 * w[k] ** 2))
        out += amp[k] * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    return out


def gaussian_rhs_box(n, seed, box, nblobs=16, wmin=0.02, wmax=0.1):
    """``gaussian_rhs(n, seed)`` on the cells of one box ((lo, hi) or a
    6-tuple lo+hi), shape (nz, ny, nx) of the box; the same values, bit for
    bit, without forming the whole-domain array."""
    n = _as3(n)
    lo, hi = (tuple(box[:3]), tuple(box[3:])) if len(box) == 6 else (tuple(box[0]), tuple(box[1]))
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(0.0, 1.0, size=(nblobs, 3))
    w = rng.uniform(wmin, wmax, size=nblobs)
    amp = rng.standard_normal(nblobs)
    x, y, z = cell_centres(n)
    x, y, z = x[lo[0]:hi[0] + 1], y[lo[1]:hi[1] + 1], z[lo[2]:hi[2] + 1]
    out = np.zeros((len(z), len(y), len(x)), dtype=np.float64)
    for k in range(nblobs):
        gx = np.exp(-((x - c[k, 0]) ** 2) / (2 * w[k] ** 2))
        gy = np.exp(-((y - c[k, 1]) ** 2) / (2 * w[k] ** 2))
        gz = np.exp(-((z - c[k, 2]) ** 2) / (2 * w[k] ** 2))
        out += amp[k] * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    return out


def gaussian_random_field(shape_zyx, seed, sigma_cells=5.0):
    """White noise convolved (periodically, via FFT) with a Gaussian of
    ``sigma_cells`` cells, normalised to zero mean and unit variance."""
    rng = np.random.Generator(np.random.PCG64(seed))
    noise = rng.standard_normal(shape_zyx)
    kz = np.fft.fftfreq(shape_zyx[0])[:, None, None]
    ky = np.fft.fftfreq(shape_zyx[1])[None, :, None]
    kx = np.fft.rfftfreq(shape_zyx[2])[None, None, :]
    # Fourier transform of a unit-mass Gaussian with std sigma (in cells)
    filt = np.exp(-2.0 * (np.pi * sigma_cells) ** 2 * (kx * kx + ky * ky + kz * kz))
    g = np.fft.irfftn(np.fft.rfftn(noise) * filt, s=shape_zyx, axes=(0, 1, 2))
    g -= g.mean()
    g /= g.std()
    return g


def lognormal_bcoef(n, seed, sigma_cells=5.0, contrast=3.0, max_ratio=None):
    """Face b-coefficients (bx, by, bz) with shapes (nz,ny,nx+1), (nz,ny+1,nx),
    (nz+1,ny,nx).

    ``b = exp(kappa * g)`` with ``kappa = contrast``; if ``max_ratio`` is
    given, kappa is instead chosen so that max(b)/min(b) over the field equals
    ``max_ratio`` exactly (kappa = ln(max_ratio) / (max g - min g))."""
    n = _as3(n)
    nx, ny, nz = n
    g = gaussian_random_field((nz + 2, ny + 2, nx + 2), seed, sigma_cells)
    kappa = contrast if max_ratio is None else np.log(max_ratio) / (g.max() - g.min())
    bcc = np.exp(kappa * g)
    bx = 0.5 * (bcc[1:-1, 1:-1, :-1] + bcc[1:-1, 1:-1, 1:])
    by = 0.5 * (bcc[1:-1, :-1, 1:-1] + bcc[1:-1, 1:, 1:-1])
    bz = 0.5 * (bcc[:-1, 1:-1, 1:-1] + bcc[1:, 1:-1, 1:-1])
    return (np.ascontiguousarray(bx), np.ascontiguousarray(by), np.ascontiguousarray(bz))


def smooth_field(n, seed, sigma_cells=5.0):
    n = _as3(n)
    return np.ascontiguousarray(gaussian_random_field((n[2], n[1], n[0]), seed, sigma_cells))


def _as3(n):
    if np.isscalar(n):
        return (int(n), int(n), int(n))
    return tuple(int(v) for v in n)
