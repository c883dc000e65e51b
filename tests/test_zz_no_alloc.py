"""ps_gpu_bin_fields_noalloc (static device scratch, no allocation on the
call path) against the allocating ps_gpu_bin_fields_host, called twice in a
row through the C ABI.  Collected last on purpose: it must hold after every
other test has run on the device, and alone."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("poles", [(0, 2, 4), (0, 1, 2, 3, 4, 5, 6)])
def test_noalloc_binning_matches_allocating_entry_point(gpu_lib, poles):
    import torch
    ng = 32
    rng = np.random.default_rng(11)
    shape = (ng, ng, ng // 2 + 1)
    f1 = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    f2 = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    L = gpu_lib.lib()
    with gpu_lib.Estimator(ng=ng, assign=3, interlace=True, dk=0.01, poles=poles) as e:
        ref = e.bin_fields(f1, f2)
        d1 = torch.from_numpy(f1.view(np.float32)).cuda()
        d2 = torch.from_numpy(f2.view(np.float32)).cuda()
        out = torch.full((len(poles) * e.nbin,), float("nan"), dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        got = []
        for _ in range(2):
            rc = L.ps_gpu_bin_fields_noalloc(e._ctx, d1.data_ptr(), d2.data_ptr(),
                                             out.data_ptr(), ctypes.c_void_p(stream))
            assert rc == 0, L.ps_gpu_last_error(e._ctx)
            torch.cuda.synchronize()
            got.append(out.cpu().numpy().reshape(len(poles), e.nbin).copy())
            out.fill_(float("nan"))
    # The binning kernel adds FP32 tile sums in shared memory (atomics, in no
    # fixed order) before flushing them to FP64 partials, and the two entry
    # points split the modes over different CTA counts: every call agrees with
    # the allocating one, and with the other call, to FP32 summation error.
    scale = np.abs(ref[0]).max()
    for g in got:
        assert np.isfinite(g).all()
        assert (np.abs(g - ref) / scale).max() <= 2e-6
    assert (np.abs(got[0] - got[1]) / scale).max() <= 2e-6


def test_noalloc_rejects_oversized_binning(gpu_lib):
    import torch
    ng = 32
    L = gpu_lib.lib()
    # dk = 2e-4 on L = 1000: ~ 540 bins x 7 poles > 3200 partial-sum columns
    with gpu_lib.Estimator(ng=ng, assign=1, dk=2e-4, poles=(0, 1, 2, 3, 4, 5, 6)) as e:
        assert 7 * e.nbin > 3200
        d = torch.zeros(ng * ng * (ng // 2 + 1) * 2, dtype=torch.float32, device="cuda")
        out = torch.zeros(7 * e.nbin, dtype=torch.float64, device="cuda")
        rc = L.ps_gpu_bin_fields_noalloc(e._ctx, d.data_ptr(), d.data_ptr(), out.data_ptr(), None)
        assert rc == -22
        assert b"scratch limit" in L.ps_gpu_last_error(e._ctx)


def test_noalloc_allocates_nothing_and_outlives_a_context(gpu_lib):
    """A warm call leaves the device's free memory unchanged, and the call
    stays correct on a context created after another one was destroyed
    (the scratch address is looked up on every call, never cached)."""
    import torch
    ng = 48
    rng = np.random.default_rng(5)
    shape = (ng, ng, ng // 2 + 1)
    f = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    L = gpu_lib.lib()
    d = torch.from_numpy(f.view(np.float32)).cuda()
    dev_before = torch.cuda.current_device()
    for _ in range(2):  # the second context is created after the first is gone
        with gpu_lib.Estimator(ng=ng, assign=2, interlace=False, dk=0.01) as e:
            ref = e.bin_fields(f)
            out = torch.zeros(3 * e.nbin, dtype=torch.float64, device="cuda")
            stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
            assert L.ps_gpu_bin_fields_noalloc(e._ctx, d.data_ptr(), d.data_ptr(),
                                               out.data_ptr(), stream) == 0
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            out.fill_(float("nan"))
            assert L.ps_gpu_bin_fields_noalloc(e._ctx, d.data_ptr(), d.data_ptr(),
                                               out.data_ptr(), stream) == 0
            torch.cuda.synchronize()
            assert torch.cuda.mem_get_info()[0] == free0, "the warm call allocated device memory"
            got = out.cpu().numpy().reshape(3, e.nbin)
            assert (np.abs(got - ref) / np.abs(ref[0]).max()).max() <= 2e-6
    assert torch.cuda.current_device() == dev_before
