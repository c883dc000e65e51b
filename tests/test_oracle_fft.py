"""The oracle's FFTW-API shim against numpy.fft (pocketfft)."""
import ctypes
import os

import numpy as np
import pytest

import oracle

SHIM = os.path.join(os.path.dirname(oracle.HERE), "oracle", "fftw_shim")


@pytest.fixture(scope="module")
def shim(oracle_mod):
    L = oracle_mod.port()
    L.fftw_plan_dft_r2c_3d.restype = ctypes.c_void_p
    L.fftw_plan_dft_c2r_3d.restype = ctypes.c_void_p
    L.fftw_execute_dft_r2c.argtypes = [ctypes.c_void_p] * 3
    L.fftw_execute_dft_c2r.argtypes = [ctypes.c_void_p] * 3
    L.fftw_destroy_plan.argtypes = [ctypes.c_void_p]
    return L


def r2c(L, x):
    n0, n1, n2 = x.shape
    out = np.zeros((n0, n1, n2 // 2 + 1), np.complex128)
    p = L.fftw_plan_dft_r2c_3d(n0, n1, n2, None, None, 0)
    L.fftw_execute_dft_r2c(p, x.ctypes.data, out.ctypes.data)
    L.fftw_destroy_plan(p)
    return out


def c2r(L, X, n2):
    n0, n1, _ = X.shape
    X = X.copy()
    out = np.zeros((n0, n1, n2))
    p = L.fftw_plan_dft_c2r_3d(n0, n1, n2, None, None, 0)
    L.fftw_execute_dft_c2r(p, X.ctypes.data, out.ctypes.data)
    L.fftw_destroy_plan(p)
    return out


@pytest.mark.parametrize("shape", [(8, 8, 8), (12, 12, 12), (30, 30, 30), (64, 64, 64),
                                   (5, 7, 9), (6, 10, 15), (16, 12, 7), (1, 1, 1), (2, 2, 2),
                                   (22, 26, 34), (128, 128, 128)])
def test_r2c_c2r_match_numpy(shim, shape):
    x = np.random.default_rng(1).standard_normal(shape)
    ref = np.fft.rfftn(x)
    got = r2c(shim, x)
    assert np.abs(got - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())
    back = c2r(shim, ref, shape[2])
    n = np.prod(shape)
    assert np.abs(back - n * x).max() <= 1e-13 * n * np.abs(x).max()


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 11, 13, 16, 17, 97, 101, 1000, 1024, 1536, 2048])
def test_cfft1d_match_numpy(shim, n):
    rng = np.random.default_rng(n)
    z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    a = z.copy()
    assert shim.ps_shim_cfft1d(n, -1, ctypes.c_void_p(a.ctypes.data)) == 0
    ref = np.fft.fft(z)
    assert np.abs(a - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())
