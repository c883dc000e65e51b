"""The oracle's C restatement against the REFERENCE compiled from source.

Needs the reference source tree (only where it is mounted); with one
OpenMP thread the restatement performs the reference's floating-point
operations in the reference's order, so every output must be bit-identical.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.skipif(oracle.build_ref() is None,
                                reason="reference sources not present")

FIELDS = ("k", "kedge", "km", "cnt", "lcnt", "pl", "xpl", "shot", "norm")


@pytest.fixture(autouse=True)
def one_thread(oracle_mod):
    oracle_mod.set_threads(1)
    yield


@pytest.mark.parametrize("assign", [0, 1, 2, 3])
@pytest.mark.parametrize("interlace", [False, True])
def test_mesh_bit_identical(assign, interlace):
    from powspec_gb300 import catalog
    cat = catalog.lognormal(4000, box=1000.0, seed=3 + assign, ngen=32, weights=(0.5, 1.5))
    mp = oracle.assign("port", cat, 16, 1000.0, assign, interlace)
    mr = oracle.assign("ref", cat, 16, 1000.0, assign, interlace)
    for a, b in zip(mp if interlace else [mp], mr if interlace else [mr]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("assign", [0, 1, 2, 3])
@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("logscale", [False, True])
def test_run_bit_identical(assign, interlace, logscale):
    from powspec_gb300 import catalog
    c1 = catalog.lognormal(3000, box=1000.0, seed=11, ngen=32)
    c2 = catalog.lognormal(3000, box=1000.0, seed=12, ngen=32)
    spec = oracle.Spec(ng=16, assign=assign, interlace=interlace, poles=(0, 1, 2, 3, 4, 5, 6),
                       dk=0.1 if logscale else 0.01, logscale=logscale,
                       kmin=np.log10(0.01) if logscale else 0.0)
    rp = oracle.run("port", spec, [c1, c2])
    rr = oracle.run("ref", spec, [c1, c2])
    for f in FIELDS:
        assert np.array_equal(getattr(rp, f), getattr(rr, f)), f


def test_reference_cli_matches_golden(tmp_path):
    """The reference CLI on the committed ASCII catalogue reproduces the golden output."""
    import os
    import shutil
    import subprocess
    src = os.path.join(os.path.dirname(__file__), "golden", "cli")
    for f in ("data.txt", "powspec.conf"):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    subprocess.run([oracle.REF_CLI, "-c", "powspec.conf"], cwd=tmp_path, check=True,
                   env=dict(os.environ, OMP_NUM_THREADS="1"), stdout=subprocess.DEVNULL)
    got = (tmp_path / "ref_auto.txt").read_text()
    ref = open(os.path.join(src, "ref_auto.txt")).read()
    assert got == ref
