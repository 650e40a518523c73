"""Device numerics of the library's own helpers."""
import ctypes

import numpy as np
import pytest

from pnepma_gb300 import capi

pytestmark = pytest.mark.gpu


def test_fp32_phi1_matches_expm1f_form(gpu_lib):
    """phi1(c) = (e^c - 1)/c in FP32 (Taylor below |c| = 1/4, fast exponential above) against
    expm1f(c)/c: relative difference within 3e-6 over the range the march produces."""
    x = np.concatenate([-np.logspace(-7, 2, 4000), np.logspace(-7, 1.5, 4000), [0.0, 0.25, -0.25]]).astype(np.float32)
    fast = np.zeros_like(x)
    ref = np.zeros_like(x)
    L = capi.lib()
    rc = L.pn_selftest_phi1(len(x), x.ctypes.data_as(ctypes.c_void_p), fast.ctypes.data_as(ctypes.c_void_p),
                            ref.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    exact = np.where(x == 0, 1.0, np.expm1(x.astype(np.float64)) / np.where(x == 0, 1.0, x.astype(np.float64)))
    assert np.max(np.abs(ref - exact) / exact) < 1e-6
    assert np.max(np.abs(fast.astype(np.float64) - ref) / np.abs(ref)) < 3e-6
