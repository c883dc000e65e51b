"""The Ng = 2048 y and x passes by pairs of warps (each 2048-point line held
by 64 lanes, 32 values each, transposed through the pair's shared memory
and finished by radix-2 butterflies between neighbouring lanes) against the
block-tiled passes: the same mode counts, and multipoles within the FP32
transform's rounding, with and without interlacing."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L = 2000.0


@pytest.mark.parametrize("interlace", [False, True])
def test_2048_pairs_match_block_tiled(gpu_lib, interlace):
    from powspec_gb300 import catalog
    cat = catalog.lognormal(2_000_000, box=L, seed=77, ngen=128, weights=(0.5, 1.5))
    out = {}
    for warp in (True, False):
        with gpu_lib.Estimator(ng=2048, box=L, assign=3, interlace=interlace, dk=0.002) as e:
            mask = e.warp_fft()
            assert mask & 6 == 6, "the Ng = 2048 y and x passes have their pair-of-warps forms"
            e.warp_fft(mask if warp else mask & ~6)
            out[warp] = e.run([cat])
    a, b = out[True], out[False]
    assert np.array_equal(a.cnt, b.cnt)
    scale = np.abs(b.pl[0][0]) + b.shot[0]
    use = b.cnt > 0
    err = (np.abs(a.pl[0] - b.pl[0])[:, use] / scale[use]).max()
    print(f"interlace={interlace}: max |dP|/(|P0|+shot) = {err:.2e}")
    assert err <= 1e-5
