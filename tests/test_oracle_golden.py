"""The oracle restatement against the golden fixtures made by the reference.

These run everywhere (the fixtures are committed); with one thread the
restatement reproduces the reference up to libm differences between
machines, and mode counts exactly.
"""
import numpy as np
import pytest

from conftest import GOLDEN, cats_of, golden_cases, spec_of

CASES = golden_cases()


@pytest.fixture(autouse=True)
def one_thread(oracle_mod):
    oracle_mod.set_threads(1)
    yield


@pytest.mark.parametrize("name", sorted(CASES))
def test_port_matches_reference_fixture(oracle_mod, name):
    case = CASES[name]
    spec = spec_of(case, oracle_mod)
    r = oracle_mod.run("port", spec, cats_of(case))
    assert r.nbin == len(case["k"])
    assert np.array_equal(r.cnt, case["cnt"])
    for f in ("k", "kedge", "shot", "norm", "lcnt"):
        np.testing.assert_allclose(getattr(r, f), case[f], rtol=1e-12, atol=1e-12, err_msg=f)
    if not spec.logscale:
        np.testing.assert_allclose(r.km, case["km"], rtol=1e-12)
    scale = np.abs(case["pl"][0, 0]) + case["shot"][0]
    assert (np.abs(r.pl - case["pl"]) / scale).max() < 1e-10
    if spec.iscross:
        assert (np.abs(r.xpl - case["xpl"]) / scale).max() < 1e-10


@pytest.mark.parametrize("assign", [0, 1, 2, 3])
def test_port_meshes_match_reference_fixture(oracle_mod, assign):
    import os
    d = np.load(os.path.join(GOLDEN, "ref_meshes.npz"))
    m0, m1 = oracle_mod.assign("port", d["cat"], 16, 1000.0, assign, True)
    np.testing.assert_allclose(m0, d[f"fr_{assign}"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(m1, d[f"frl_{assign}"], rtol=0, atol=1e-12)
