"""Stage-level parity: assignment mesh, FFT and binning, each in isolation."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

MESH_RTOL = 2e-7  # of the largest cell (FP32 node products)


@pytest.mark.parametrize("assign", [0, 1, 2, 3])
def test_mesh_matches_reference_fixture(gpu_lib, assign):
    d = np.load(os.path.join(GOLDEN, "ref_meshes.npz"))
    with gpu_lib.Estimator(ng=16, assign=assign, interlace=True, dk=0.01) as e:
        e.assign(0, d["cat"])
        m0, m1 = e.read_mesh(0, 0), e.read_mesh(0, 1)
    # Each node value is an FP32 product of the 1-D weights (~4 roundings,
    # ~2.4e-7 relative) rounded to 2^-32 units; the mesh total then matches
    # sum(w) to that relative rounding (only the unused k = 0 mode sees it).
    for got, ref in ((m0, d[f"fr_{assign}"]), (m1, d[f"frl_{assign}"])):
        assert np.abs(got - ref).max() <= MESH_RTOL * np.abs(ref).max()
        assert got.sum() == pytest.approx(ref.sum(), rel=1e-7)


@pytest.mark.parametrize("assign", [0, 1, 2, 3])
@pytest.mark.parametrize("interlace", [False, True])
def test_mesh_matches_oracle_and_is_deterministic(gpu_lib, oracle_mod, assign, interlace):
    from powspec_gb300 import catalog
    cat = catalog.lognormal(200000, box=1000.0, seed=8, ngen=64, weights=(0.5, 1.5))
    ref = oracle_mod.assign("port", cat, 48, 1000.0, assign, interlace)
    ref = ref if interlace else (ref,)
    with gpu_lib.Estimator(ng=48, assign=assign, interlace=interlace, dk=0.01) as e:
        runs = []
        for _ in range(2):
            e.assign(0, cat)
            runs.append([e.read_mesh(0, m) for m in range(2 if interlace else 1)])
    for m in range(len(ref)):
        assert np.array_equal(runs[0][m], runs[1][m]), "mesh not bit-reproducible"
        assert np.abs(runs[0][m] - ref[m]).max() <= MESH_RTOL * np.abs(ref[m]).max()


@pytest.mark.parametrize("ng,warp", [(n, False) for n in (8, 12, 16, 20, 24, 30, 32, 40, 48, 60, 64,
                                                     96, 128, 192, 256)] + [(256, True), (512, True),
                                                                            (512, False)])
def test_fft_r2c_matches_numpy(gpu_lib, ng, warp):
    """warp: the warp-register z and y passes (ps_wfft.cu) where the size has
    them, else the block-tiled passes."""
    x = np.random.default_rng(ng).standard_normal((ng, ng, ng)).astype(np.float32)
    with gpu_lib.Estimator(ng=ng, dk=2 * np.pi / 1000) as e:
        m = e.warp_fft(7 if warp else 0)
        assert bool(m & 3) == (warp and ng >= 256)
        got = e.fft_r2c(x)
    ref = np.fft.rfftn(x.astype(np.float64))
    # FP32 transform: error ~ eps * log2(n) * ||x||_2
    bound = 6e-8 * np.log2(ng ** 3) * np.sqrt((x.astype(np.float64) ** 2).sum())
    assert np.abs(got - ref).max() <= bound


@pytest.mark.parametrize("assign,interlace", [(1, False), (3, False), (2, True)])
def test_binning_alone_matches_oracle(gpu_lib, oracle_mod, assign, interlace):
    import ctypes
    from powspec_gb300 import catalog
    ng = 32
    poles = (0, 1, 2, 3, 4, 5, 6)
    cat = catalog.lognormal(30000, box=1000.0, seed=5, ngen=32)
    spec = oracle_mod.Spec(ng=ng, assign=assign, interlace=interlace, dk=0.01, poles=poles)
    m = oracle_mod.assign("port", cat, ng, 1000.0, assign, False)
    fk = oracle_mod.r2c(m)
    alias, cnt, km = oracle_mod.precomp(spec)
    kedge, _ = oracle_mod.bins(spec)
    nb = len(kedge) - 1
    pl = np.zeros((7, nb))
    lc = np.zeros((7, nb))
    oracle_mod.port().ps_oracle_count_sim(
        ng, (ctypes.c_double * 3)(1000., 1000., 1000.), oracle_mod._ptr(alias), oracle_mod._ptr(fk),
        oracle_mod._ptr(fk), 0, nb, oracle_mod._ptr(kedge), ctypes.c_double(0.01),
        (ctypes.c_double * 3)(0, 0, 1.), 7, (ctypes.c_int * 7)(*poles), oracle_mod._ptr(pl),
        oracle_mod._ptr(lc))
    with gpu_lib.Estimator(ng=ng, assign=assign, interlace=interlace, dk=0.01, poles=poles) as e:
        got = e.bin_fields(fk.astype(np.complex64))
    assert (np.abs(got - pl) / np.abs(pl[0])).max() <= 2e-6


def _host_gb():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 2 ** 20
    except OSError:
        pass
    return 0.0


@pytest.mark.parametrize("ng", [512, 1024])
def test_fft_r2c_matches_cufft(gpu_lib, ng):
    """The hand-written r2c (z, y and x passes) against cuFFT, called through
    torch.fft.rfftn on the same FP32 cube (the reference's transform is
    FFTW's r2c, src/fftw_define.h:56, called at src/multipole.c:444,459).
    cuFFT in FP64 is the truth; the FP32 error of ours must be within a
    norm-scaled bound and at most twice cuFFT's own FP32 error."""
    torch = pytest.importorskip("torch")
    need = 4 * ng ** 3 * 3.2 / 2 ** 30
    if _host_gb() < need + 8:
        pytest.skip(f"needs about {need:.0f} GB of host memory")
    g = torch.Generator(device="cuda").manual_seed(ng)
    xd = torch.randn((ng, ng, ng), device="cuda", dtype=torch.float32, generator=g)
    x = xd.cpu().numpy()
    with gpu_lib.Estimator(ng=ng, dk=2 * np.pi / 1000) as e:
        got = e.fft_r2c(x)
    ref64 = torch.fft.rfftn(xd.double())
    cu32 = torch.fft.rfftn(xd)
    gd = torch.from_numpy(got).cuda()
    del got
    err = (gd.to(torch.complex128) - ref64).abs()
    err_cu = (cu32.to(torch.complex128) - ref64).abs()
    norm = torch.sqrt((xd.double() ** 2).sum()).item()
    emax, ecu_max = err.max().item(), err_cu.max().item()
    rms = torch.sqrt((err ** 2).mean()).item()
    rms_cu = torch.sqrt((err_cu ** 2).mean()).item()
    print(f"ng={ng}: max |ours - fp64| = {emax:.3e}, cuFFT fp32 {ecu_max:.3e}; "
          f"rms {rms:.3e} vs cuFFT {rms_cu:.3e}; ||x|| = {norm:.3e}")
    assert emax <= 6e-8 * np.log2(ng ** 3) * norm
    assert rms <= 2.0 * rms_cu
