"""The large single-mesh configuration (L = 2000 Mpc/h, float32 positions and
weights in [0.5, 1.5], PCS interlaced, dk = 0.002) at Ng = 1024 and 2048,
where the FP64 reference does not fit in host memory.  Size-independent
checks: (1) mode counts bit-exact against an independent host count of the
lattice (1-D square histograms convolved, k = 0 / Nyquist planes weighted
1, the rest 2, and each |k|^2 binned with the reference's FP64 rule,
src/multipole.c:111-257; the few |k|^2 within rounding of a bin edge are
enumerated decomposition by decomposition, as the reference sums them);
(2) a uniform catalogue's multipoles equal the estimator's weighted
shot-noise residual (P_0) and zero (P_2, P_4) within their statistical
error."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOX, DK = 2000.0, 0.002


def ref_bin(kmod, kedge, dk):
    if kmod < kedge[0] or kmod >= kedge[-1]:
        return -1
    b = int((kmod - kedge[0]) / dk)
    return b if 0 <= b < len(kedge) - 1 else -1


def host_counts(ng, kedge):
    h = ng // 2
    vec = 2 * math.pi / BOX
    s1 = np.full(h + 1, 2.0)
    s1[0] = s1[h] = 1.0          # |i'| = 0 and ng/2 occur once, the rest twice
    wk = np.full(h + 1, 2.0)
    wk[0] = wk[h] = 1.0          # k = 0 and Nyquist planes weigh 1
    nmax = 3 * h * h
    a = np.zeros(h * h + 1)
    a[np.arange(h + 1) ** 2] = s1
    kk = np.zeros(h * h + 1)
    kk[np.arange(h + 1) ** 2] = wk
    size = 1 << int(np.ceil(np.log2(nmax + 1)))
    fa, fk = np.fft.rfft(a, size), np.fft.rfft(kk, size)
    mult = np.rint(np.fft.irfft(fa * fa * fk, size)[:nmax + 1])
    nb = len(kedge) - 1
    cnt = np.zeros(nb, np.int64)
    n = np.nonzero(mult)[0]
    t = n * (vec * vec)
    kmod = np.sqrt(t)
    lo = (kmod * (1 - 1e-12) - kedge[0]) / DK
    hi = (kmod * (1 + 1e-12) - kedge[0]) / DK
    inside = (kmod * (1 - 1e-12) >= kedge[0]) & (kmod * (1 + 1e-12) < kedge[-1])
    outside = (kmod * (1 + 1e-12) < kedge[0]) | (kmod * (1 - 1e-12) >= kedge[-1])
    clear = inside & (np.floor(lo) == np.floor(hi))
    b = np.floor(lo[clear]).astype(np.int64)
    ok = (b >= 0) & (b < nb)
    np.add.at(cnt, b[ok], mult[n[clear]][ok].astype(np.int64))
    # within rounding of a bin edge or of the range ends: the reference's FP64
    # expression per decomposition ((kx^2 + ky^2) + kz^2)
    ksq = [(m * vec) * (m * vec) for m in range(h + 1)]
    for nn in n[~clear & ~outside]:
        for c in range(h + 1):
            r2 = nn - c * c
            if r2 < 0:
                break
            for x in range(min(h, math.isqrt(r2)) + 1):
                y2 = r2 - x * x
                y = math.isqrt(y2)
                if y * y != y2 or y > h:
                    continue
                km = math.sqrt((ksq[x] + ksq[y]) + ksq[c])
                bb = ref_bin(km, kedge, DK)
                if bb >= 0:
                    cnt[bb] += int(s1[x] * s1[y] * wk[c])
    return cnt


@pytest.mark.parametrize("ng,n", [(1024, 20_000_000), (2048, 150_000_000)])
def test_large_mesh_counts_and_uniform_field(gpu_lib, ng, n):
    rng = np.random.default_rng(ng)
    x, y, z = (rng.random(n, dtype=np.float32) * np.float32(BOX) for _ in range(3))
    for v in (x, y, z):
        np.minimum(v, np.nextafter(np.float32(BOX), np.float32(0)), out=v)
    w = (rng.random(n, dtype=np.float32) + np.float32(0.5)).astype(np.float32)
    with gpu_lib.Estimator(ng=ng, box=BOX, assign=3, interlace=True, dk=DK) as e:
        e.assign(0, x=x, y=y, z=z, w=w)
        r = e.execute()
    assert r.wdata[0] == pytest.approx(float(np.sum(w, dtype=np.float64)), rel=1e-12)
    ref = host_counts(ng, r.kedge)
    assert np.array_equal(r.cnt.astype(np.int64), ref)
    # Uniform field: the white-noise level of weighted particles is
    # V sum(w^2) / W^2, while the estimator subtracts V / W
    # (src/genr_mesh.c:907): P_0 = shot (sum(w^2) / W - 1), P_l>0 = 0, up to
    # noise of std ~ shot * sqrt((2l+1) / (cnt/2)); the aliased shot noise
    # stays small below 0.3 k_Nyq
    w64 = w.astype(np.float64)
    expect0 = r.shot[0] * (np.sum(w64 * w64) / np.sum(w64) - 1.0)
    kny = math.pi * ng / BOX
    use = (r.k < 0.3 * kny) & (r.cnt > 200)
    for li, ell in enumerate(e.poles):
        sig = r.shot[0] * np.sqrt((2 * ell + 1) / (r.cnt[use] / 2.0))
        expect = expect0 if ell == 0 else 0.0
        assert (np.abs(r.pl[0][li][use] - expect) <= 6 * sig + 0.01 * r.shot[0]).all(), ell
