"""Why the GPU sums F_l(0) in FP64: the estimator's arithmetic done in FP32
with NumPy/SciPy (FP32 meshes, harmonics and transforms, FP64 bin sums),
against the oracle's FP64 survey path, for the cross of two catalogues in
one box.

* Each catalogue's n(z) consistent between its data and randoms: the
  weighted field's total W = F(k = 0) is about 0, and every bin is within
  1e-5 of |P_0| + the noise scale.
* A second catalogue (a subsample) that keeps the full sample's n(z) while
  its randoms keep their own: W is 8.6% of its sum of |w|, and the first
  bin (k = 0 alone) is dominated by W F_l(0), where
  F_l(0) = sum_m sum_r F Y_lm(r^) cancels to a small part of its terms.
  That bin exceeds 1e-5 in FP32 while every other bin stays within it.
* With the k = 0 term taken as the GPU takes it, W (the weight sum) times
  F_l(0) summed over the mesh in FP64, harmonics included, that bin is
  within 1e-5 as well.  (FP32 harmonics, 1e-7 off each, are not enough:
  that bin is W F_l(0), many times the noise scale.)
"""
import numpy as np
import pytest

import oracle
from powspec_gb300 import catalog

sf = pytest.importorskip("scipy.fft")

NG = 64


def _pair(unbalanced):
    d1, r1 = catalog.survey(50000, seed=11)
    _, r2 = catalog.survey(40000, seed=12)
    d2 = d1[np.random.default_rng(3).random(len(d1)) < 0.6].copy()
    r2 = r2.copy()
    if not unbalanced:  # else the subsample keeps the full sample's n(z)
        d2[:, 4] *= 0.6
        r2[:, 4] = d2[0, 4]
    return catalog.prepare_survey([(d1, r1), (d2, r2)])


def _ylm32(l, m, x, y, z):
    """The real harmonic of the estimator's basis, in FP32."""
    f32 = np.float32
    x, y, z = x.astype(f32), y.astype(f32), z.astype(f32)
    rxy2 = x * x + y * y
    r = np.sqrt(rxy2 + z * z)
    ct, st = z / r, np.sqrt(rxy2) / r
    am = abs(m)
    fac = 1.0
    for q in range(l - am + 1, l + am + 1):
        fac /= q
    kl = f32(np.sqrt((2 * l + 1) / (4 * np.pi) * fac) * (np.sqrt(2.0) if m else 1.0))
    pmm = np.ones_like(x)
    for i in range(1, am + 1):
        pmm = pmm * f32(2 * i - 1) * st
    p = pmm
    if l > am:
        p0, p1 = pmm, ct * f32(2 * am + 1) * pmm
        p = p1
        for ll in range(am + 2, l + 1):
            p = (f32(2 * ll - 1) * ct * p1 - f32(ll + am - 1) * p0) / f32(ll - am)
            p0, p1 = p1, p
    if m == 0:
        return kl * p
    with np.errstate(invalid="ignore", divide="ignore"):
        ri = f32(1) / np.sqrt(rxy2)
    cp, sp = x * ri, y * ri
    c, s = np.ones_like(x), np.zeros_like(x)
    for _ in range(am):
        c, s = c * cp - s * sp, s * cp + c * sp
    return kl * p * (c if m > 0 else s)


def _ylm64(l, m, x, y, z):
    """The same harmonic in FP64 (the GPU's F_l(0) sum)."""
    rxy2 = x * x + y * y
    r = np.sqrt(rxy2 + z * z)
    ct, st = z / r, np.sqrt(rxy2) / r
    am = abs(m)
    fac = 1.0
    for q in range(l - am + 1, l + am + 1):
        fac /= q
    kl = np.sqrt((2 * l + 1) / (4 * np.pi) * fac) * (np.sqrt(2.0) if m else 1.0)
    pmm = np.ones_like(x)
    for i in range(1, am + 1):
        pmm = pmm * (2 * i - 1) * st
    p = pmm
    if l > am:
        p0, p1 = pmm, ct * (2 * am + 1) * pmm
        p = p1
        for ll in range(am + 2, l + 1):
            p = ((2 * ll - 1) * ct * p1 - (ll + am - 1) * p0) / (ll - am)
            p0, p1 = p1, p
    if m == 0:
        return kl * p
    with np.errstate(invalid="ignore", divide="ignore"):
        ri = 1.0 / np.sqrt(rxy2)
    cp, sp = x * ri, y * ri
    c, s = np.ones_like(x), np.zeros_like(x)
    for _ in range(am):
        c, s = c * cp - s * sp, s * cp + c * sp
    return kl * p * (c if m > 0 else s)


def _fp32_cross(cats, want, alias, poles, dc64=False):
    ngk = NG // 2 + 1
    L = np.array(cats[0].box)
    o = cats[0].origin * NG / L
    i, j, k = np.meshgrid(np.arange(NG), np.arange(NG), np.arange(NG), indexing="ij")
    X, Y, Z = (i + o[0]) * L[0], (j + o[1]) * L[1], (k + o[2]) * L[2]
    fi = np.fft.fftfreq(NG, 1.0 / NG)
    KI, KJ, KK = np.meshgrid(fi / L[0], fi / L[1], np.arange(ngk) / L[2], indexing="ij")
    axis = (KI == 0) & (KJ == 0)
    kmod = 2 * np.pi * np.sqrt(KI ** 2 + KJ ** 2 + KK ** 2)
    wmode = np.where((np.arange(ngk) == 0) | (2 * np.arange(ngk) == NG), 1.0, 2.0)[None, None, :]
    use = alias != 0
    b = ((kmod - want.kedge[0]) / 0.01).astype(int)[use]

    def count(f1, f2):
        v = (f1.real.astype(np.float64) * f2.real + f1.imag.astype(np.float64) * f2.imag)
        return np.bincount(b, weights=(v * wmode * alias)[use], minlength=want.nbin)[:want.nbin]

    meshes = [oracle.assign("port", c.xyzw, NG, tuple(L), 3, False).astype(np.float32) for c in cats]
    f0 = [sf.rfftn(m) for m in meshes]
    wsum = [float(c.xyzw[:, 3].sum()) for c in cats]
    b0 = int((0.0 - want.kedge[0]) / 0.01)

    def k0_term(f1, f2):
        return float(f1.real) * float(f2.real) + float(f1.imag) * float(f2.imag)

    out = np.zeros((len(poles), want.nbin))
    for li, l in enumerate(poles):
        if l == 0:
            out[li] = count(f0[0], f0[1])
            continue
        fl, dcl = [], []
        for c in range(2):
            acc = np.zeros((NG, NG, ngk), np.complex64)
            ysum = np.zeros((NG, NG, NG))
            for m in range(-l, l + 1):
                y = _ylm32(l, m, X, Y, Z)
                y[0, 0, :] = 1
                if dc64:
                    with np.errstate(invalid="ignore", divide="ignore"):
                        y64 = _ylm64(l, m, X.astype(np.float64), Y.astype(np.float64),
                                     Z.astype(np.float64))
                    y64[0, 0, :] = 1
                    ysum += y64
                with np.errstate(invalid="ignore", divide="ignore"):
                    yk = _ylm32(l, m, KI, KJ, KK)
                acc += sf.rfftn(meshes[c] * y) * np.where(axis, np.float32(1), yk)
            fl.append(acc)
            dcl.append(float(np.sum(meshes[c].astype(np.float64) * ysum)))
        out[li] = count(f0[0], fl[1]) + count(f0[1], fl[0])
        if dc64 and alias[0, 0, 0] != 0 and 0 <= b0 < want.nbin:
            # the k = 0 mode as W_a F_l,b(0) + W_b F_l,a(0), both factors FP64
            fp32 = k0_term(f0[0][0, 0, 0], fl[1][0, 0, 0]) + k0_term(f0[1][0, 0, 0], fl[0][0, 0, 0])
            out[li, b0] += (wsum[0] * dcl[1] + wsum[1] * dcl[0] - fp32) * alias[0, 0, 0]
    norm = np.sqrt(cats[0].norm * cats[1].norm) * np.maximum(want.cnt, 1)
    for li, l in enumerate(poles):
        out[li] *= (2 * np.pi if l else 1.0) / norm
    return out


@pytest.mark.parametrize("unbalanced", [False, True])
def test_fp32_cross_error_is_confined_to_the_k0_bin(unbalanced):
    poles = (0, 2, 4)
    cats = _pair(unbalanced)
    spec = oracle.Spec(ng=NG, box=cats[0].box, assign=3, interlace=False, poles=poles, dk=0.01,
                       isauto=(False, False), iscross=True)
    want = oracle.survey(spec, [c.xyzw for c in cats], cats[0].origin,
                         [c.shot for c in cats], [c.norm for c in cats])
    alias, _, _ = oracle.precomp(spec)
    got = _fp32_cross(cats, want, alias, poles)
    scale = np.abs(want.xpl[0]) + np.sqrt(cats[0].shot / cats[0].norm * cats[1].shot / cats[1].norm)
    use = want.cnt > 0
    err = np.abs(got - want.xpl)[:, use] / scale[use]
    assert err[:, 1:].max() <= 1e-5, err[:, 1:].max(axis=1)
    if unbalanced:
        assert abs(cats[1].xyzw[:, 3].sum()) > 0.05 * np.abs(cats[1].xyzw[:, 3]).sum()
        assert 1e-5 < err[:, 0].max() <= 2e-4, err[:, 0]
    else:
        assert err[:, 0].max() <= 1e-5, err[:, 0]


def test_fp64_k0_term_keeps_every_bin_within_1e5():
    """The unbalanced pair again, with the k = 0 term formed as the GPU forms
    it: every bin, the first included, is within 1e-5."""
    poles = (0, 2, 4)
    cats = _pair(True)
    spec = oracle.Spec(ng=NG, box=cats[0].box, assign=3, interlace=False, poles=poles, dk=0.01,
                       isauto=(False, False), iscross=True)
    want = oracle.survey(spec, [c.xyzw for c in cats], cats[0].origin,
                         [c.shot for c in cats], [c.norm for c in cats])
    alias, _, _ = oracle.precomp(spec)
    got = _fp32_cross(cats, want, alias, poles, dc64=True)
    scale = np.abs(want.xpl[0]) + np.sqrt(cats[0].shot / cats[0].norm * cats[1].shot / cats[1].norm)
    use = want.cnt > 0
    err = np.abs(got - want.xpl)[:, use] / scale[use]
    assert err.max() <= 1e-5, err.max(axis=1)
