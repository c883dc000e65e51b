"""The region gather (each TSC/PCS record added once, into its home tile's
region, then the regions summed per cell) against the tile gather (each tile
replays the records that reach it, one per warp or in lane groups): the
fixed-point meshes (int64 regions) are the same to the bit, for particles on
the box faces, across the interlaced grid's periodic wrap, with weights large
enough for the 64-bit node conversion, and with most tiles empty.  The FP32
meshes the spectra use sum FP32 regions, a few FP32 roundings per cell, so
their spectra are compared within the FP32 binning bar."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L = 1000.0


def _catalogue(n, ng, seed, heavy=True):
    from powspec_gb300 import catalog
    cat = catalog.lognormal(n, box=L, seed=seed, ngen=32, weights=(0.5, 1.5))
    rng = np.random.default_rng(seed)
    # faces, cell edges and half-cell edges (the shifted grid's edges)
    top = np.nextafter(L, 0.0)
    edge = np.array([0.0, top, L / ng, L - L / ng, 0.5 * L / ng, L - 0.5 * L / ng, 1e-9, L - 1e-9])
    k = 4000
    extra = np.empty((k, 4))
    for a in range(3):
        extra[:, a] = rng.choice(edge, k)
        mix = rng.random(k) < 0.3
        extra[mix, a] = rng.random(mix.sum()) * L
    extra[:, 3] = rng.uniform(0.5, 1.5, k)
    if heavy:
        extra[:50, 3] = 4000.0  # node values above 2^31 in 2^-32 units
    return np.concatenate([cat, extra])


def _run(gpu_lib, cat, ng, assign, interlace, region, lanes=False):
    with gpu_lib.Estimator(ng=ng, box=L, assign=assign, interlace=interlace, dk=0.02) as e:
        e.set_tuning(region_gather=region, dense_lane_groups=lanes)
        e.assign(0, cat)
        meshes = [e.read_mesh(0, m) for m in range(2 if interlace else 1)]
        spec = e.execute()
    return meshes, spec


@pytest.mark.parametrize("ng", [32, 64])
@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("assign", [2, 3])
def test_region_gather_equals_tile_gather(gpu_lib, assign, interlace, ng):
    cat = _catalogue(60000, ng, seed=ng + assign)
    mr, sr = _run(gpu_lib, cat, ng, assign, interlace, True)
    mt, st = _run(gpu_lib, cat, ng, assign, interlace, False)
    ml, _ = _run(gpu_lib, cat, ng, assign, interlace, False, lanes=True)
    for a, b, c in zip(mr, mt, ml):
        assert np.array_equal(a, b)
        assert np.array_equal(a, c)  # lane groups on every tile
    assert np.array_equal(sr.cnt, st.cnt)
    scale = np.abs(st.pl[0][0]) + st.shot[0]
    use = st.cnt > 0
    # the same FP32 mesh; the binning's FP32 sums may add in another order,
    # and its mu^2 moments (P_4 = 4.375 M_2 - 3.75 M_1 + 0.375 M_0) carry
    # that order's rounding into P_l at a few 1e-7 of the monopole
    assert (np.abs(sr.pl[0] - st.pl[0])[:, use] / scale[use]).max() <= 5e-6


def test_region_gather_with_empty_tiles(gpu_lib):
    """Particles in one corner: most tiles have no record, and their stale
    regions from the previous catalogue must not reach the mesh."""
    ng = 64
    full = _catalogue(80000, ng, seed=3, heavy=False)
    corner = full[(full[:, 0] < 200) & (full[:, 1] < 300) & (full[:, 2] < 150)]
    with gpu_lib.Estimator(ng=ng, box=L, assign=3, interlace=True, dk=0.02) as e:
        e.set_tuning(region_gather=True)
        e.assign(0, full)
        e.execute()
        e.assign(0, corner)
        got = [e.read_mesh(0, m) for m in range(2)]
    ref, _ = _run(gpu_lib, corner, ng, 3, True, False)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
