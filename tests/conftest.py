"""Shared test setup.

Markers: ``gpu`` -- needs a GB300 (run with ``-m gpu``); everything else runs
on a CPU-only machine.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build_port()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree if needed; its product path must load."""
    import powspec_gb300 as ps
    if not os.path.exists(ps.LIB_PATH):
        ps.build()
    return ps


def golden_cases():
    d = np.load(os.path.join(GOLDEN, "ref_cases.npz"))
    names = sorted({k.split("/")[0] for k in d.files})
    out = {}
    for n in names:
        out[n] = {k.split("/", 1)[1]: d[k] for k in d.files if k.startswith(n + "/")}
    return out


def spec_of(case, oracle):
    ng, a, il, dk, lg, kmin, kmax, ncat = case["settings"]
    box = tuple(case["box"])
    return oracle.Spec(ng=int(ng), box=box, assign=int(a), interlace=bool(il),
                       poles=tuple(int(p) for p in case["poles"]), los=tuple(case["los"]),
                       kmin=float(kmin), kmax=float(kmax), dk=float(dk), logscale=bool(lg),
                       isauto=(True, True), iscross=int(ncat) == 2)


def cats_of(case):
    return [case[f"cat{j}"] for j in range(2) if f"cat{j}" in case]


def perr(got, ref, shot):
    """Max |P_l^got - P_l^ref| relative to the raw monopole P_0 + shot of each bin."""
    scale = np.abs(ref[0]) + shot
    return float((np.abs(np.asarray(got) - np.asarray(ref)) / scale).max())


def xerr(got, ref, pl_ref, shot):
    """Cross-spectrum error relative to sqrt of the two raw auto monopoles
    (the Cauchy-Schwarz bound on |P_cross|): the cross of independent
    catalogues is ~0, so its FP32 round-off scales with the autos."""
    scale = np.sqrt((np.abs(pl_ref[0][0]) + shot[0]) * (np.abs(pl_ref[1][0]) + shot[1]))
    return float((np.abs(np.asarray(got) - np.asarray(ref)) / scale).max())
