"""Analytic known-answer tests of the oracle (the reference ships none).

Assignment weights against the closed forms of the schemes
(src/genr_mesh.c:98-108, :157-173, :263-270), weight conservation, the
binning of a single Fourier mode, and shot-noise removal on a uniform
Poisson sample.
"""
import ctypes

import numpy as np
import pytest


def kernel_1d(assign, s):
    s = abs(s)
    if assign == 0:
        return 1.0 if s < 0.5 else 0.0
    if assign == 1:
        return max(0.0, 1 - s)
    if assign == 2:
        return 0.75 - s * s if s < 0.5 else (0.5 * (1.5 - s) ** 2 if s < 1.5 else 0.0)
    return (4 - 6 * s * s + 3 * s ** 3) / 6 if s < 1 else ((2 - s) ** 3 / 6 if s < 2 else 0.0)


@pytest.mark.parametrize("assign", [0, 1, 2, 3])
@pytest.mark.parametrize("frac", [(0.0, 0.0, 0.0), (0.5, 0.25, 0.75), (0.3, 0.9, 0.1)])
def test_single_particle_weights(oracle_mod, assign, frac):
    ng, L = 16, 16.0
    pos = np.array([[5 + frac[0], 9 + frac[1], 15 + frac[2], 2.5]])
    m = oracle_mod.assign("port", pos, ng, L, assign, False)
    exp = np.zeros((ng, ng, ng))
    for i in range(ng):
        for j in range(ng):
            for k in range(ng):
                w = 2.5
                for d, node in enumerate((i, j, k)):
                    s = node - pos[0, d]
                    s = (s + ng / 2) % ng - ng / 2  # periodic distance
                    w *= kernel_1d(assign, s)
                exp[i, j, k] = w
    if assign == 0:
        # NGP rounds up at d >= 0.5 exactly like the reference
        assert m.sum() == pytest.approx(2.5)
        assert np.count_nonzero(m) == 1
    else:
        np.testing.assert_allclose(m, exp, atol=1e-13)


@pytest.mark.parametrize("assign", [0, 1, 2, 3])
@pytest.mark.parametrize("interlace", [False, True])
def test_weight_conservation(oracle_mod, assign, interlace):
    from powspec_gb300 import catalog
    cat = catalog.uniform(5000, box=1000.0, seed=9, weights=(0.5, 1.5))
    ms = oracle_mod.assign("port", cat, 16, 1000.0, assign, interlace)
    for m in (ms if interlace else [ms]):
        assert m.sum() == pytest.approx(cat[:, 3].sum(), rel=1e-12)


def test_single_mode_lands_in_one_bin(oracle_mod):
    ng = 32
    spec = oracle_mod.Spec(ng=ng, assign=1, dk=0.01)
    alias, cnt, km = oracle_mod.precomp(spec)
    kedge, _ = oracle_mod.bins(spec)
    nb = len(kedge) - 1
    f = np.zeros((ng, ng, ng // 2 + 1), np.complex128)
    f[3, 4, 5] = 1 + 2j
    pl = np.zeros((1, nb))
    lc = np.zeros((1, nb))
    L = oracle_mod.port()
    L.ps_oracle_count_sim(ng, (ctypes.c_double * 3)(1000., 1000., 1000.), oracle_mod._ptr(alias),
                          oracle_mod._ptr(f), oracle_mod._ptr(f), 0, nb, oracle_mod._ptr(kedge),
                          ctypes.c_double(0.01), (ctypes.c_double * 3)(0, 0, 1.), 1,
                          (ctypes.c_int * 7)(0), oracle_mod._ptr(pl), oracle_mod._ptr(lc))
    kmod = 2 * np.pi / 1000 * np.sqrt(9 + 16 + 25)
    b = int(kmod / 0.01)
    assert np.count_nonzero(pl) == 1 and pl[0, b] == pytest.approx(5 * 2 * alias[3, 4, 5])


def test_uniform_poisson_shot_noise_removed(oracle_mod):
    from powspec_gb300 import catalog
    cat = catalog.uniform(200000, box=1000.0, seed=21)
    spec = oracle_mod.Spec(ng=32, assign=2, interlace=True, dk=0.02, isauto=(True, False),
                           iscross=False)
    r = oracle_mod.run("port", spec, [cat])
    sig = r.shot[0] * np.sqrt(2.0 / np.maximum(r.cnt, 1))
    ok = r.cnt > 50
    assert np.all(np.abs(r.pl[0, 0][ok]) < 6 * sig[ok] + 0.02 * r.shot[0])
