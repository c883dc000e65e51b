"""The oracle's survey path (data minus alpha x randoms, FKP weights, k = 0
binned, multipoles l > 0 by the spherical-harmonic decomposition, with and
without interlacing) against the reference's own outputs for the survey
fixture (tests/golden/survey/, written by the reference program).

The catalogue preparation restates the reference's (src/read_cata.c:95-185,
src/genr_mesh.c:509-566): w = wc x wfkp, alpha = sum wc_d / sum wc_r,
shot = sum w_d^2 + alpha^2 sum w_r^2, norm = alpha sum_r wc wfkp^2 nz, the
box centred on the bounds of data and randoms with the extent x (1 + 0.02)
rounded up to 10."""
import math
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
SURVEY = os.path.join(HERE, "golden", "survey")


def _prepare(pairs, pad=0.02):
    """(data, randoms) row pairs -> catalogues in one box fitted to all."""
    pos = np.concatenate([a[:, :3] for pr in pairs for a in pr])
    mn, mx = pos.min(axis=0), pos.max(axis=0)
    box = np.array([math.ceil((mx[a] - mn[a]) * (1 + pad) / 10) * 10 for a in range(3)])
    bmin = (mx + mn - box) * 0.5
    cats, shots, norms = [], [], []
    fkp = lambda a: 1.0 / (1.0 + a[:, 4] * 2000)
    for d, r in pairs:
        wd, wr = d[:, 3] * fkp(d), r[:, 3] * fkp(r)
        alpha = d[:, 3].sum() / r[:, 3].sum()
        shots.append((wd * wd).sum() + alpha * alpha * (wr * wr).sum())
        norms.append(alpha * (r[:, 3] * fkp(r) ** 2 * r[:, 4]).sum())
        p = np.concatenate([d[:, :3], r[:, :3]])
        cats.append(np.column_stack([p - bmin, np.concatenate([wd, -alpha * wr])]))
    return cats, bmin, tuple(box), shots, norms


def _load(name):
    return np.loadtxt(os.path.join(SURVEY, name))


def prepare(ncat=1, pad=0.02, rand_nz=1.0):
    """rand_nz: the randoms' n(z) as this multiple of the file's column."""
    d, r = _load("data.txt"), _load("rand.txt")
    r[:, 4] *= rand_nz
    return _prepare([(d, r)] * ncat, pad)


def read_ref(name):
    rows = np.array([[float(v) for v in l.split()] for l in open(os.path.join(SURVEY, name))
                     if not l.startswith("#")])
    return rows


@pytest.mark.parametrize("ref,interlace,poles,cross,rand_nz", [
    ("ref_auto.txt", True, (0,), False, 1.0),
    ("ref_auto_yama.txt", False, (0, 2, 4), False, 1.0),
    ("ref_auto_yama_il.txt", True, (0, 1, 2, 3, 4, 5, 6), False, 1.0),
    ("ref_cross_yama.txt", False, (0, 2, 4), True, 1.0),
    ("ref_auto_yama_nz.txt", True, (0, 2, 4), False, 1.5),  # F(k = 0) far from 0
])
def test_oracle_survey_matches_reference_output(ref, interlace, poles, cross, rand_nz):
    cats, bmin, box, shot, norm = prepare(2 if cross else 1, rand_nz=rand_nz)
    if rand_nz != 1.0:
        assert abs(cats[0][:, 3].sum()) > 1e-3 * np.abs(cats[0][:, 3]).sum()
    spec = oracle.Spec(ng=32, box=box, assign=3, interlace=interlace, poles=poles, dk=0.02,
                       isauto=(not cross, not cross), iscross=cross)
    res = oracle.survey(spec, cats, bmin, shot, norm)
    want = read_ref(ref)
    assert res.nbin == len(want)
    assert np.array_equal(res.cnt, want[:, 4].astype(np.uint64))
    assert np.allclose(res.km, want[:, 3], rtol=1e-9, atol=0)
    got = res.xpl if cross else res.pl[0]
    scale = np.abs(want[:, 5]) + (0.0 if cross else shot[0] / norm[0])
    err = np.abs(got.T - want[:, 5:]) / scale[:, None]
    assert err.max() <= 1e-8, err.max()


def test_oracle_survey_cross_of_two_catalogues():
    """The catalogue crossed with a 60% subsample of it and half the
    randoms, interlaced, l = 0, 2, 4 (ref_cross2_il.txt)."""
    cats, bmin, box, shot, norm = _prepare([(_load("data.txt"), _load("rand.txt")),
                                            (_load("data2.txt"), _load("rand2.txt"))])
    spec = oracle.Spec(ng=32, box=box, assign=3, interlace=True, poles=(0, 2, 4), dk=0.02,
                       isauto=(False, False), iscross=True)
    res = oracle.survey(spec, cats, bmin, shot, norm)
    want = read_ref("ref_cross2_il.txt")
    assert res.nbin == len(want)
    assert np.array_equal(res.cnt, want[:, 4].astype(np.uint64))
    err = np.abs(res.xpl.T - want[:, 5:]) / np.abs(want[:, 5:6])
    assert err.max() <= 1e-8, err.max()


def test_oracle_survey_log_bins():
    """Log-scale bins (KMIN 0.01, 0.1 dex), interlaced, l = 0, 2, 4: counts,
    the k columns with the reference's rescaling, and P_l
    (ref_auto_log.txt)."""
    cats, bmin, box, shot, norm = prepare()
    spec = oracle.Spec(ng=32, box=box, assign=3, interlace=True, poles=(0, 2, 4),
                       kmin=math.log10(0.01), dk=0.1, logscale=True, isauto=(True, False),
                       iscross=False)
    res = oracle.survey(spec, cats, bmin, shot, norm)
    want = read_ref("ref_auto_log.txt")
    assert res.nbin == len(want)
    assert np.array_equal(res.cnt, want[:, 4].astype(np.uint64))
    assert np.allclose(res.k, want[:, 0], rtol=1e-9, atol=0)
    assert np.allclose(res.km, want[:, 3], rtol=1e-9, atol=0)
    scale = np.abs(want[:, 5]) + shot[0] / norm[0]
    err = np.abs(res.pl[0].T - want[:, 5:]) / scale[:, None]
    assert err.max() <= 1e-8, err.max()


def test_ylm_orthonormal_and_addition_theorem():
    """The real harmonics are orthonormal on the sphere and satisfy
    sum_m Y_lm(a) Y_lm(b) = (2l + 1) / (4 pi) L_l(a . b)."""
    rng = np.random.default_rng(5)
    # quadrature on the sphere: Gauss-Legendre in cos t x uniform in phi
    xg, wg = np.polynomial.legendre.leggauss(16)
    ph = np.arange(32) * 2 * np.pi / 32
    ct, p = np.meshgrid(xg, ph, indexing="ij")
    st = np.sqrt(1 - ct ** 2)
    w = np.outer(wg, np.full(32, 2 * np.pi / 32))

    def Y(l, m):
        return np.vectorize(oracle.ylm)(l, m, ct, st, np.cos(p), np.sin(p))

    basis = [(l, m) for l in range(7) for m in range(-l, l + 1)]
    vals = {lm: Y(*lm) for lm in basis}
    for a in basis[::3]:
        for b in basis[::2]:
            g = (vals[a] * vals[b] * w).sum()
            assert abs(g - (a == b)) < 1e-12, (a, b, g)
    for _ in range(20):
        u, v = rng.normal(size=3), rng.normal(size=3)
        u, v = u / np.linalg.norm(u), v / np.linalg.norm(v)
        for l in range(7):
            s = 0.0
            for m in range(-l, l + 1):
                ya = oracle.ylm(l, m, u[2], math.hypot(u[0], u[1]), u[0] / math.hypot(u[0], u[1]),
                                u[1] / math.hypot(u[0], u[1]))
                yb = oracle.ylm(l, m, v[2], math.hypot(v[0], v[1]), v[0] / math.hypot(v[0], v[1]),
                                v[1] / math.hypot(v[0], v[1]))
                s += ya * yb
            want = (2 * l + 1) / (4 * np.pi) * oracle.port().ps_oracle_legpoly(l, float(u @ v))
            assert abs(s - want) < 1e-12


@pytest.mark.parametrize("rand_nz", [1.0, 1.5])
def test_prepare_survey_matches_restatement(rand_nz):
    """The package's survey preparation (used by the Python API and the
    survey workload) gives this file's restatement of the reference's:
    records, box, corner, shot noise and normalisation."""
    from powspec_gb300 import catalog
    d = np.loadtxt(os.path.join(SURVEY, "data.txt"))
    r = np.loadtxt(os.path.join(SURVEY, "rand.txt"))
    r[:, 4] *= rand_nz
    s = catalog.prepare_survey([(d, r)])[0]
    cats, bmin, box, shot, norm = prepare(rand_nz=rand_nz)
    assert np.array_equal(s.xyzw, cats[0])
    assert np.array_equal(s.origin, bmin) and s.box == box
    assert s.shot == shot[0] and s.norm == norm[0]
    # a given box: centred on the same bounds; too small is refused
    t = catalog.prepare_survey([(d, r)], box=(450.0, 420.0, 430.0))[0]
    assert t.box == (450.0, 420.0, 430.0)
    pos = np.concatenate([d[:, :3], r[:, :3]])
    assert np.allclose(t.origin, (pos.min(0) + pos.max(0) - np.array(t.box)) / 2, rtol=0, atol=1e-12)
    with pytest.raises(ValueError):
        catalog.prepare_survey([(d, r)], box=100.0)


def test_synthetic_survey_is_seeded():
    from powspec_gb300 import catalog
    a = catalog.survey(20000, seed=4)
    b = catalog.survey(20000, seed=4)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    d, r = a
    assert len(r) == 3 * len(d) and d.shape[1] == r.shape[1] == 5
    cen = np.array([600.0, 300.0, 450.0])
    for p in (d, r):
        assert np.all(np.linalg.norm(p[:, :3] - cen, axis=1) < 200.0)
