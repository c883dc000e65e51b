"""Seeded synthetic periodic-box catalogues (the reference ships none).

* ``uniform``: positions uniform in [0, L)^3.
* ``lognormal``: a Gaussian field with P(k) = A k^-1.5 exp(-(k/0.5)^2)
  normalised to unit variance, the lognormal density 1 + delta =
  exp(G - sigma^2/2), Poisson-sampled per cell with positions uniform inside
  the cell, then displaced along z by the Zel'dovich displacement of G
  (psi_z(k) = i k_z / k^2 G(k)) for redshift-space-like anisotropy.

Outputs are float64 [N, 4] records (x, y, z, w), the reference DATA layout,
or float32 SoA arrays.
"""
from __future__ import annotations

import numpy as np


def uniform(n, box=1000.0, seed=1, weights=None, dtype=np.float64):
    rng = np.random.default_rng(seed)
    out = np.empty((int(n), 4), dtype=dtype)
    out[:, :3] = rng.random((int(n), 3)) * box
    if weights is None:
        out[:, 3] = 1.0
    else:
        lo, hi = weights
        out[:, 3] = rng.uniform(lo, hi, int(n))
    np.clip(out[:, :3], 0, np.nextafter(np.array(box, dtype), 0), out=out[:, :3])
    return out


def gaussian_field(ngen, box, seed, slope=-1.5, kcut=0.5):
    """Unit-variance Gaussian field on an ngen^3 grid and its Fourier modes."""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((ngen, ngen, ngen)).astype(np.float32)
    wk = np.fft.rfftn(white)
    kf = 2 * np.pi / box
    kx = np.fft.fftfreq(ngen, 1.0 / ngen).astype(np.float32) * kf
    kz = np.fft.rfftfreq(ngen, 1.0 / ngen).astype(np.float32) * kf
    k2 = kx[:, None, None] ** 2 + kx[None, :, None] ** 2 + kz[None, None, :] ** 2
    k = np.sqrt(k2)
    with np.errstate(divide="ignore"):
        amp = np.where(k > 0, k ** (slope / 2) * np.exp(-0.5 * (k / kcut) ** 2), 0.0)
    gk = wk * amp.astype(np.float32)
    g = np.fft.irfftn(gk, s=(ngen, ngen, ngen), axes=(0, 1, 2)).astype(np.float32)
    s = g.std()
    g /= s
    gk /= s
    return g, gk, kz, k2


def lognormal(nbar_total, box=1000.0, seed=1, ngen=128, zeldovich=4.0, weights=None,
              dtype=np.float64, soa=False):
    """Poisson sample of ~nbar_total points from a lognormal field.

    zeldovich: rms displacement (Mpc/h) along z added to every particle.
    """
    g, gk, kz, k2 = gaussian_field(ngen, box, seed)
    dens = np.exp(g - 0.5)  # sigma_G^2 = 1
    rng = np.random.default_rng(seed + 7919)
    cell = box / ngen
    lam = dens.ravel() * (nbar_total / dens.size) / dens.mean()
    counts = rng.poisson(lam)
    n = int(counts.sum())
    idx = np.repeat(np.arange(dens.size, dtype=np.int64), counts)
    ix, rem = np.divmod(idx, ngen * ngen)
    iy, iz = np.divmod(rem, ngen)
    pos = np.empty((n, 3), dtype=np.float64)
    pos[:, 0] = (ix + rng.random(n)) * cell
    pos[:, 1] = (iy + rng.random(n)) * cell
    pos[:, 2] = (iz + rng.random(n)) * cell
    if zeldovich:
        with np.errstate(divide="ignore", invalid="ignore"):
            psik = np.where(k2 > 0, 1j * kz[None, None, :] / k2, 0) * gk
        psi = np.fft.irfftn(psik, s=(ngen, ngen, ngen), axes=(0, 1, 2)).astype(np.float32)
        psi *= zeldovich / max(psi.std(), 1e-30)
        pos[:, 2] += psi.ravel()[idx]
    pos %= box
    np.clip(pos, 0, np.nextafter(box, 0), out=pos)
    if weights is None:
        w = np.ones(n)
    else:
        w = rng.uniform(weights[0], weights[1], n)
    if soa:
        # FP32 rounding may reach L itself: keep every coordinate below it
        top = np.nextafter(np.float32(box), np.float32(0))
        xyz = [np.minimum(pos[:, a].astype(np.float32), top) for a in range(3)]
        return xyz[0], xyz[1], xyz[2], w.astype(np.float32)
    out = np.empty((n, 4), dtype=dtype)
    out[:, :3] = pos
    out[:, 3] = w
    return out
