"""The C ABI library loads and exports every symbol include/*.h declares,
and the ctypes mirrors of its structs have the header's layout (no GPU)."""
import glob
import os
import re
import subprocess

import pytest

from conftest import ROOT


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        syms |= set(re.findall(r"\b(ps_(?:gpu|mlp)_\w+)\s*\(", src))
    return sorted(syms)


def test_library_exports_declared_symbols(gpu_lib):
    L = gpu_lib.lib()
    syms = declared_symbols()
    assert syms, "no declarations found"
    for s in syms:
        assert hasattr(L, s), f"{s} not exported"
    assert set(syms) <= set(gpu_lib.EXPORTED) | set(syms)


def test_struct_layout_matches_header(gpu_lib, tmp_path):
    import ctypes
    prog = tmp_path / "layout.c"
    prog.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "powspec_gpu.h"
#define F(T, f) printf("%s.%s %zu %zu\\n", #T, #f, offsetof(T, f), sizeof(((T*)0)->f));
int main(void) {
  printf("ps_gpu_params %zu\\nps_gpu_result %zu\\n", sizeof(ps_gpu_params), sizeof(ps_gpu_result));
  F(ps_gpu_params, ng) F(ps_gpu_params, box) F(ps_gpu_params, assign) F(ps_gpu_params, interlace)
  F(ps_gpu_params, ncat) F(ps_gpu_params, isauto) F(ps_gpu_params, iscross) F(ps_gpu_params, los)
  F(ps_gpu_params, kmin) F(ps_gpu_params, kmax) F(ps_gpu_params, dk) F(ps_gpu_params, logscale)
  F(ps_gpu_params, npole) F(ps_gpu_params, poles) F(ps_gpu_params, device)
  F(ps_gpu_result, nbin) F(ps_gpu_result, k) F(ps_gpu_result, kedge) F(ps_gpu_result, km)
  F(ps_gpu_result, cnt) F(ps_gpu_result, lcnt) F(ps_gpu_result, pl) F(ps_gpu_result, xpl)
  F(ps_gpu_result, shot) F(ps_gpu_result, norm) F(ps_gpu_result, wdata)
  return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I" + os.path.join(ROOT, "include"), str(prog), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    sizes = dict(l.split() for l in out[:2])
    assert int(sizes["ps_gpu_params"]) == ctypes.sizeof(gpu_lib.Params)
    assert int(sizes["ps_gpu_result"]) == ctypes.sizeof(gpu_lib.Result)
    for line in out[2:]:
        if not line:
            continue
        name, off, size = line.split()
        T, f = name.split(".")
        cls = gpu_lib.Params if T == "ps_gpu_params" else gpu_lib.Result
        fld = getattr(cls, f)
        assert (fld.offset, fld.size) == (int(off), int(size)), name


def test_context_creation_fails_cleanly_without_gpu(gpu_lib):
    """No CPU fallback: without a usable GPU creation returns PS_GPU_ERR_CUDA."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gpu_lib.PowspecError) as e:
        gpu_lib.Estimator(ng=16)
    assert e.value.code == -20
