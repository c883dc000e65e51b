"""Seeded synthetic periodic-box catalogues (the reference ships none).

* ``uniform``: positions uniform in [0, L)^3.
* ``lognormal``: a Gaussian field with P(k) = A k^-1.5 exp(-(k/0.5)^2)
  normalised to unit variance, the lognormal density 1 + delta =
  exp(G - sigma^2/2), Poisson-sampled per cell with positions uniform inside
  the cell, then displaced along z by the Zel'dovich displacement of G
  (psi_z(k) = i k_z / k^2 G(k)) for redshift-space-like anisotropy.

Outputs are float64 [N, 4] records (x, y, z, w), the reference DATA layout,
or float32 SoA arrays.

Surveys (``survey``, ``prepare_survey``): a lognormal sample cut to a sphere
and uniform randoms in the same sphere, with completeness weights and a
constant n(z); then the reference's survey preparation (src/read_cata.c:
95-185, src/genr_mesh.c:509-566) into the catalogue the survey path takes.
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
              dtype=np.float64, soa=False, sample_seed=None):
    """Poisson sample of ~nbar_total points from a lognormal field.

    zeldovich: rms displacement (Mpc/h) along z added to every particle.
    sample_seed: seed of the Poisson sampling (default seed + 7919); two
    samples of one field (the same `seed`) differ only in it.
    """
    g, gk, kz, k2 = gaussian_field(ngen, box, seed)
    dens = np.exp(g - 0.5)  # sigma_G^2 = 1
    rng = np.random.default_rng(seed + 7919 if sample_seed is None else sample_seed)
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


def survey(ndata, centre=(600.0, 300.0, 450.0), radius=200.0, nrand=3, seed=1, ngen=64):
    """Synthetic survey: about `ndata` lognormal points in a sphere (data)
    and nrand x as many uniform points in the same sphere (randoms).  Each
    row is (x, y, z, wcomp, nz): completeness weights uniform in [0.8, 1.2]
    and the data's mean density as n(z)."""
    cen = np.asarray(centre, dtype=np.float64)
    side = 2.0 * radius
    c = lognormal(ndata * 6.0 / np.pi, box=side, seed=seed, ngen=ngen)[:, :3] - radius
    d = c[np.einsum("ij,ij->i", c, c) < radius * radius] + cen
    rng = np.random.default_rng(seed + 104729)
    want = nrand * len(d)
    r = np.empty((0, 3))
    while len(r) < want:
        u = rng.uniform(-radius, radius, (int(want * 2.0) + 1024, 3))
        r = np.concatenate([r, u[np.einsum("ij,ij->i", u, u) < radius * radius]])
    r = r[:want] + cen
    nbar = len(d) / (4.0 / 3.0 * np.pi * radius ** 3)
    out = []
    for pts in (d, r):
        out.append(np.column_stack([pts, rng.uniform(0.8, 1.2, len(pts)), np.full(len(pts), nbar)]))
    return out[0], out[1]


class SurveyCatalogue:
    """What the survey path takes for one catalogue: xyzw = data (weight
    wc wfkp) then randoms (weight -alpha wc wfkp), positions minus the box
    corner `origin`; shot noise and normalisation (src/read_cata.c:165-183)."""

    def __init__(self, xyzw, origin, box, alpha, shot, norm):
        self.xyzw, self.origin, self.box = xyzw, origin, box
        self.alpha, self.shot, self.norm = alpha, shot, norm


def prepare_survey(pairs, p0=2000.0, box=None, pad=0.02):
    """(data, randoms) pairs of (x, y, z, wcomp, nz) rows -> one
    SurveyCatalogue per pair, in a common box: FKP weights 1 / (1 + nz p0),
    alpha = sum wc_d / sum wc_r, shot = sum w_d^2 + alpha^2 sum w_r^2,
    norm = alpha sum_r wc wfkp^2 nz (sum_d when the randoms' is 0); the box
    centred on the bounds of every data and random point, `box` or the
    extent x (1 + pad) rounded up to 10 (src/genr_mesh.c:509-566)."""
    pts = np.concatenate([a[:, :3] for pr in pairs for a in pr])
    mn, mx = pts.min(axis=0), pts.max(axis=0)
    if box is None:
        size = np.array([np.ceil((mx[a] - mn[a]) * (1 + pad) / 10) * 10 for a in range(3)])
    else:
        size = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)).copy()
        if np.any(mx - mn > size):
            raise ValueError("box smaller than the catalogues' extent")
    origin = (mx + mn - size) * 0.5
    out = []
    for d, r in pairs:
        fd, fr = 1.0 / (1.0 + d[:, 4] * p0), 1.0 / (1.0 + r[:, 4] * p0)
        wd, wr = d[:, 3] * fd, r[:, 3] * fr
        alpha = d[:, 3].sum() / r[:, 3].sum()
        shot = (wd * wd).sum() + alpha * alpha * (wr * wr).sum()
        sd, sr = (d[:, 3] * fd * fd * d[:, 4]).sum(), (r[:, 3] * fr * fr * r[:, 4]).sum()
        norm = alpha * sr if (sd == 0 or sr != 0) else sd
        xyzw = np.empty((len(d) + len(r), 4))
        xyzw[:len(d), :3] = d[:, :3] - origin
        xyzw[len(d):, :3] = r[:, :3] - origin
        xyzw[:len(d), 3] = wd
        xyzw[len(d):, 3] = -alpha * wr
        out.append(SurveyCatalogue(xyzw, origin, tuple(float(x) for x in size), alpha, shot, norm))
    return out
