"""The oracle's CPU FFT (backing both the oracle and the FFTW-subset shim of the reference build) against numpy."""
import ctypes
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def cfft():
    import subprocess
    out = os.path.join(ROOT, "oracle", "_build", "libcfft_test.so")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-o", out, os.path.join(ROOT, "oracle", "cfft.c"), "-lm"],
                   check=True)
    L = ctypes.CDLL(out)
    return L


class Plan(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("nf", ctypes.c_int), ("fac", ctypes.c_int * 64), ("tw", ctypes.c_void_p)]


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8, 11, 12, 13, 16, 20, 22, 26, 30, 32, 36, 40, 48, 60, 64, 96,
                               98, 128, 192, 256, 350, 512])
@pytest.mark.parametrize("sign", [-1, 1])
def test_cfft_vs_numpy(cfft, n, sign):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    p = Plan()
    assert cfft.cfft_plan_init(ctypes.byref(p), n) == 0
    d = x.copy()
    w = np.empty_like(d)
    cfft.cfft_exec(ctypes.byref(p), d.ctypes.data_as(ctypes.c_void_p), w.ctypes.data_as(ctypes.c_void_p), sign)
    ref = np.fft.fft(x) if sign < 0 else np.fft.ifft(x) * n
    assert np.max(np.abs(d - ref)) <= 1e-13 * np.max(np.abs(ref)) * max(1, np.log2(n))
    cfft.cfft_plan_free(ctypes.byref(p))
