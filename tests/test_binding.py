"""The reference-side binding (powspec_gb300/binding/gpu_path.c): the
reference's own main, load_conf, read_cata, cnvt_coord and save_res,
compiled unmodified from the reference tree, with genr_mesh / powspec /
mesh_destroy / powspec_destroy taken from the binding on top of the C ABI
(src/powspec.c:47,55; src/genr_mesh.h:86; src/multipole.h:78).

The binary is built where the reference tree exists (`make -C oracle
binding`); elsewhere these tests skip.  Without a GPU the reference's main
runs up to the first GPU call and takes its own error exit
(POWSPEC_ERR_MESH); with one, its output file matches the reference's own
output for the same catalogue.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

MESH_EXIT = 256 - 13  # POWSPEC_ERR_MESH (src/define.h:120) as an exit status


@pytest.fixture(scope="module")
def binding_exe():
    import oracle
    ref = oracle.ref_dir()
    if not ref or not os.path.isdir(os.path.join(ref, "src")):
        pytest.skip("the reference tree is not on this machine")
    from powspec_gb300 import buildlib
    buildlib.build_lib()
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "binding", f"REF={ref}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = os.path.join(ROOT, "oracle", "_ref", "POWSPEC_GPU")
    assert os.path.exists(exe)
    return exe


def _workdir(tmp_path):
    for f in ("data.txt", "powspec.conf"):
        shutil.copy(os.path.join(GOLDEN, "cli", f), tmp_path / f)
    return tmp_path


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_binding_links_the_reference_objects(binding_exe):
    r = subprocess.run(["nm", "-D", "--undefined-only", binding_exe], capture_output=True, text=True)
    undefined = r.stdout
    for sym in ("ps_gpu_create", "ps_gpu_assign_aos", "ps_gpu_execute", "ps_gpu_destroy"):
        assert sym in undefined, f"{sym} not bound to libpowspec_gpu.so"
    r = subprocess.run(["nm", binding_exe], capture_output=True, text=True)
    for sym in ("load_conf", "read_cata", "save_res", "genr_mesh", "powspec"):
        assert f" T {sym}\n" in r.stdout, sym


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU exit path")
def test_binding_without_gpu_takes_the_reference_error_exit(binding_exe, tmp_path):
    wd = _workdir(tmp_path)
    r = subprocess.run([binding_exe, "-c", "powspec.conf", "-a", "out.txt"], cwd=wd,
                       capture_output=True, text=True, timeout=120)
    out = r.stdout + r.stderr
    assert r.returncode == MESH_EXIT, out
    assert "Reading catalogs" in out and "no CUDA device" in out
    assert not (wd / "out.txt").exists()


@pytest.mark.gpu
def test_binding_output_matches_reference(binding_exe, tmp_path):
    if not _has_gpu():
        pytest.skip("needs a GPU")
    wd = _workdir(tmp_path)
    r = subprocess.run([binding_exe, "-c", "powspec.conf", "-a", "out.txt"], cwd=wd,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got = open(wd / "out.txt").read().splitlines()
    ref = open(os.path.join(GOLDEN, "cli", "ref_auto.txt")).read().splitlines()
    assert [l for l in got if l.startswith("#")] == [l for l in ref if l.startswith("#")]
    g = np.loadtxt(wd / "out.txt")
    f = np.loadtxt(os.path.join(GOLDEN, "cli", "ref_auto.txt"))
    np.testing.assert_array_equal(g[:, :5], f[:, :5])
    scale = np.abs(f[:, 5]) + 1.0
    assert (np.abs(g[:, 5:] - f[:, 5:]) / scale[:, None]).max() <= 1e-5
