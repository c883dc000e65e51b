"""The warp-register x pass (transform + combine + binning) against the
block-tiled one on the same meshes, at the sizes with a warp form:

* line of sight along z, one spectrum: the +-k_y form, which bins the lines
  ky and Ng - ky together (4-warp CTAs);
* line of sight along x: the unpaired warp form;
* two catalogues with their cross spectrum: the unpaired form, three spectra;
* 16 |mu| sub-bins at Ng = 256: the +-k_y form in 16-warp CTAs.

Both read the same FP32 meshes and run transforms of the same lengths; the
FP32 tile sums add in other orders, so the bar is 2e-6 of |P_0| + shot."""
import numpy as np
import pytest

from conftest import perr, xerr

pytestmark = pytest.mark.gpu
TOL = 2e-6


def _cats(n, k):
    from powspec_gb300 import catalog
    return [catalog.lognormal(n, box=1000.0, seed=11 + s, ngen=64) for s in range(k)]


def _run(ps, cats, ng, los, warp, nmu=1):
    with ps.Estimator(ng=ng, box=1000.0, assign=3, interlace=True, ncat=len(cats), los=los,
                      dk=0.005) as e:
        mask = e.warp_fft()
        assert mask & 4, "no warp x pass at this size"
        e.warp_fft(mask if warp else mask & ~4)
        if nmu > 1:
            e.set_mu_bins(nmu)
        r = e.run(cats)
        kmu = e.read_kmu(1) if nmu > 1 else None
    return r, kmu


@pytest.mark.parametrize("ng", [256, 512])
@pytest.mark.parametrize("los", [(0.0, 0.0, 1.0), (1.0, 0.0, 0.0)])
def test_warp_x_pass_matches_block_tiled(gpu_lib, ng, los):
    cats = _cats(200000, 1)
    w, _ = _run(gpu_lib, cats, ng, los, True)
    b, _ = _run(gpu_lib, cats, ng, los, False)
    assert np.array_equal(w.cnt, b.cnt)
    assert perr(w.pl[0], b.pl[0], b.shot[0]) <= TOL


def test_warp_x_pass_cross_matches_block_tiled(gpu_lib):
    cats = _cats(150000, 2)
    w, _ = _run(gpu_lib, cats, 256, (0.0, 0.0, 1.0), True)
    b, _ = _run(gpu_lib, cats, 256, (0.0, 0.0, 1.0), False)
    assert np.array_equal(w.cnt, b.cnt)
    for c in range(2):
        assert perr(w.pl[c], b.pl[c], b.shot[c]) <= TOL
    assert xerr(w.xpl, b.xpl, b.pl, b.shot) <= TOL


def test_warp_x_pass_mu_bins_match_block_tiled(gpu_lib):
    """The (k, |mu|) sums of the 16-warp form against the block-tiled pass,
    each relative to its k bin's monopole sum over |mu|."""
    cats = _cats(200000, 1)
    _, kw = _run(gpu_lib, cats, 256, (0.0, 0.0, 1.0), True, nmu=16)
    _, kb = _run(gpu_lib, cats, 256, (0.0, 0.0, 1.0), False, nmu=16)
    scale = np.abs(kb[0, 0]).sum(axis=-1)[None, :, None]
    use = scale[0, :, 0] > 0
    err = (np.abs(kw[0] - kb[0]) / np.where(scale > 0, scale, 1.0))[:, use]
    assert err.max() <= TOL, err.max()
