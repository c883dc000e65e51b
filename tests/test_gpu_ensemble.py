"""Mock ensembles: catalogues of uneven size, mesh and scheme evaluated
through one ensemble CUDA graph (ps_gpu_ensemble_*) over per-context graphs
(ps_gpu_batch_*) after autotuning (ps_gpu_autotune), against one-at-a-time
evaluations in fresh contexts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cats(torch):
    from powspec_gb300 import catalog
    specs = [(20000, 1), (5000, 2), (60000, 3), (12000, 4), (30000, 5), (800, 6)]
    cats = [catalog.lognormal(n, box=1000.0, seed=s, ngen=32) for n, s in specs]
    return cats, [torch.from_numpy(c).cuda() for c in cats]


CONFIGS = [(32, 1, True), (48, 2, True), (32, 1, True), (64, 2, True), (48, 2, True), (32, 3, False)]


def test_ensemble_matches_single_evaluations(gpu_lib):
    torch = pytest.importorskip("torch")
    from powspec_gb300.ensemble import Ensemble
    cats, dev = _cats(torch)
    ens = Ensemble(dev, CONFIGS, dk=0.01)
    try:
        assert set(ens.tuning) == set(CONFIGS)
        for t in ens.tuning.values():
            assert t["gather_threads"] in (256, 512)
        got = ens.run()
        again = ens.run()  # replay of the same graphs
        assert ens.launches() > 0
    finally:
        ens.close()
    for cat, cf, g, g2 in zip(cats, CONFIGS, got, again):
        ng, assign, il = cf
        with gpu_lib.Estimator(ng=ng, assign=assign, interlace=il, dk=0.01) as e:
            e.assign(0, cat)
            ref = e.execute()
        assert np.array_equal(g.cnt, ref.cnt)
        assert g.wdata[0] == pytest.approx(ref.wdata[0], rel=1e-12)
        scale = np.abs(ref.pl[0][0]) + ref.shot[0]
        use = ref.cnt > 0
        for x in (g, g2):
            assert (np.abs(x.pl[0] - ref.pl[0])[:, use] / scale[use]).max() <= 5e-6


def test_empty_catalogue_in_a_batch(gpu_lib):
    torch = pytest.importorskip("torch")
    from powspec_gb300 import catalog
    c = torch.from_numpy(catalog.lognormal(4000, box=1000.0, seed=3, ngen=32)).cuda()
    with gpu_lib.Estimator(ng=32, assign=1, interlace=True, dk=0.01) as e:
        b = e.batch([c.data_ptr(), c.data_ptr()], [c.shape[0], 0])
        try:
            b.launch()
            r0 = b.result(0)
            assert r0.cnt.sum() > 0
            with pytest.raises(gpu_lib.PowspecError) as ei:
                b.result(1)
            assert ei.value.code == -11
        finally:
            b.close()


def test_group_split_over_lanes(gpu_lib):
    """One configuration's catalogues split over several contexts (lanes)
    whose graphs run concurrently inside the ensemble graph: the same
    results as the per-context graph launches and as single evaluations."""
    torch = pytest.importorskip("torch")
    from powspec_gb300 import catalog
    from powspec_gb300.ensemble import Ensemble
    cats = [catalog.lognormal(8000 + 3000 * s, box=1000.0, seed=40 + s, ngen=32) for s in range(8)]
    dev = [torch.from_numpy(c).cuda() for c in cats]
    cfg = [(48, 2, True)] * 8
    ens = Ensemble(dev, cfg, dk=0.01, lanes=3, min_per_lane=2)
    try:
        assert len(ens.lanes) == 3
        got = ens.run()
        ens.launch_groups()
        ens.wait_groups()
        again = ens.results()
    finally:
        ens.close()
    for cat, g, g2 in zip(cats, got, again):
        with gpu_lib.Estimator(ng=48, assign=2, interlace=True, dk=0.01) as e:
            e.assign(0, cat)
            ref = e.execute()
        assert np.array_equal(g.cnt, ref.cnt)
        scale = np.abs(ref.pl[0][0]) + ref.shot[0]
        use = ref.cnt > 0
        for x in (g, g2):
            assert (np.abs(x.pl[0] - ref.pl[0])[:, use] / scale[use]).max() <= 5e-6
