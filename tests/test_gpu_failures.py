"""Failure paths, made on the host (no GPU fault, no device hang).

Out-of-memory: the reference allocates its meshes inside an OpenMP region
and calls exit(POWSPEC_ERR_MEMORY) when an allocation fails
(src/multipole.c:121-126).  Here every allocation failure is reported as
PS_GPU_ERR_MEMORY by the entry point that hit it, the process goes on, and
the library stays usable.  The failure comes from a fake of the failing
call (ps_gpu_debug_fail_alloc), which never calls CUDA for that
allocation.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MEMORY = -1


def _small_cat():
    from powspec_gb300 import catalog
    return catalog.lognormal(20000, box=1000.0, seed=3, ngen=32)


@pytest.fixture
def fail_alloc(gpu_lib):
    L = gpu_lib.lib()
    yield L.ps_gpu_debug_fail_alloc
    L.ps_gpu_debug_fail_alloc(0)


@pytest.mark.parametrize("nth", [1, 2, 5, 9, 14])
def test_create_reports_out_of_memory(gpu_lib, fail_alloc, nth):
    fail_alloc(nth)
    with pytest.raises(gpu_lib.PowspecError) as ei:
        gpu_lib.Estimator(ng=32, assign=3, interlace=True, dk=0.01)
    assert ei.value.code == MEMORY
    assert "out of memory" in str(ei.value)
    fail_alloc(0)
    cat = _small_cat()
    with gpu_lib.Estimator(ng=32, assign=3, interlace=True, dk=0.01) as e:
        r = e.run([cat])
    assert r.cnt.sum() > 0 and np.isfinite(r.pl).all()


def test_assign_reports_out_of_memory_and_recovers(gpu_lib, oracle_mod, fail_alloc):
    cat = _small_cat()
    with gpu_lib.Estimator(ng=32, assign=1, interlace=True, dk=0.01) as e:
        for nth in (1, 2):  # the rank buffer, then the record buffer
            fail_alloc(nth)
            with pytest.raises(gpu_lib.PowspecError) as ei:
                e.assign(0, cat)
            assert ei.value.code == MEMORY
        fail_alloc(0)
        r = e.run([cat])  # the same context, after the failures
    spec = oracle_mod.Spec(ng=32, assign=1, interlace=True, dk=0.01, isauto=(True, False),
                           iscross=False)
    ref = oracle_mod.run("port", spec, [cat])
    assert np.array_equal(r.cnt, ref.cnt)
    scale = np.abs(ref.pl[0, 0]) + ref.shot[0]
    assert (np.abs(r.pl[0] - ref.pl[0]) / scale).max() <= 1e-5


def test_bounded_wait_runs_out_and_the_context_recovers(gpu_lib, oracle_mod):
    """The bulk-copy pipelines' barrier waits are bounded: with one copy
    armed but never issued (ps_gpu_debug_stall_pipeline) and a short poll
    limit, the wait runs out, the kernel drains its other copy and stops,
    and the evaluation reports PS_GPU_ERR_CUDA -- no fault, no hang.  The
    next evaluation on the same context is correct."""
    cat = _small_cat()
    spec = oracle_mod.Spec(ng=256, assign=3, interlace=True, dk=0.01, isauto=(True, False),
                           iscross=False)
    ref = oracle_mod.run("port", spec, [cat])
    L = gpu_lib.lib()
    with gpu_lib.Estimator(ng=256, assign=3, interlace=True, dk=0.01) as e:
        e.warp_fft(0)                      # the bulk-copy pipelined passes
        e.set_tuning(pipelined_pass_c=True)
        assert L.ps_gpu_debug_stall_pipeline(e._ctx, 2048) == 0
        e.assign(0, cat)
        with pytest.raises(gpu_lib.PowspecError) as ei:
            e.execute()
        assert ei.value.code == -20 and "timed out" in str(ei.value)
        r = e.run([cat])
    assert np.array_equal(r.cnt, ref.cnt)
    scale = np.abs(ref.pl[0, 0]) + ref.shot[0]
    assert (np.abs(r.pl[0] - ref.pl[0]) / scale).max() <= 1e-5
