"""Staged input (ps_gpu_stage_aos / ps_gpu_assign_staged): catalogues copied
into two device slots on a copy stream, each copy overlapping the
evaluation before it, give the results of plain assign + execute."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cats():
    from powspec_gb300 import catalog
    sizes = [30000, 80000, 5000, 120000]  # growing and shrinking slots
    return [catalog.lognormal(n, box=1000.0, seed=40 + i, ngen=32) for i, n in enumerate(sizes)]


def test_stream_matches_single_evaluations(gpu_lib):
    torch = pytest.importorskip("torch")
    cats = [torch.from_numpy(c).pin_memory().numpy() for c in _cats()]
    with gpu_lib.Estimator(ng=64, assign=3, interlace=True, dk=0.01) as e:
        got = list(e.run_stream(cats))
        ref = []
        for c in cats:
            e.assign(0, c)
            ref.append(e.execute())
    assert len(got) == len(cats)
    for g, r in zip(got, ref):
        assert np.array_equal(g.cnt, r.cnt)
        assert g.wdata[0] == r.wdata[0]
        scale = np.abs(r.pl[0][0]) + r.shot[0]
        use = r.cnt > 0
        assert (np.abs(g.pl[0] - r.pl[0])[:, use] / scale[use]).max() <= 5e-6


@pytest.mark.parametrize("ng,lanes", [(128, 1), (256, 1), (256, 2)])
def test_learned_stream_matches_run(gpu_lib, ng, lanes):
    """Ng = 256 PCS: no fine-mesh fallback, so the stream enqueues each next
    copy and assignment before the previous results are waited for."""
    torch = pytest.importorskip("torch")
    from powspec_gb300 import learned
    cats = [torch.from_numpy(c).pin_memory().numpy() for c in _cats()[:3]]
    with learned.LearnedEstimator(ng=ng, assign=3, interlace=True) as le:
        if ng == 256:
            assert le.fine is None
        got = list(le.run_stream(cats, lanes=lanes))
        ref = [le.run(c) for c in cats]
    for (k1, p1, t1), (k2, p2, t2) in zip(got, ref):
        assert np.array_equal(k1, k2) and np.array_equal(t1, t2)
        # the binning's FP32 sums may add in another order from run to run
        assert (np.abs(p1 - p2) / np.abs(p2[0]).max()).max() <= 5e-6


def test_assign_from_an_empty_slot_fails(gpu_lib):
    with gpu_lib.Estimator(ng=32, assign=1, dk=0.01) as e:
        with pytest.raises(gpu_lib.PowspecError) as ei:
            e.assign_staged(0, 1)
        assert ei.value.code == -21  # PS_GPU_ERR_STATE
