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


def test_fp64_phi1_matches_expm1_form(gpu_lib):
    """phi1(c) = (e^c - 1)/c in FP64 on the device (the reference's Taylor form below |c| = 2e-4,
    series of 7 to 15 terms chosen by |c| up to 0.7, the exponential form beyond) against
    expm1(c)/c, which is good to an ulp or two: within the reference form's own truncation
    |c|^3/24 below 2e-4 and 6e-15 above, on both sides of every range boundary."""
    edges = np.array([2e-4, 0.03, 0.1, 0.3, 0.7])
    near = np.concatenate([edges * f for f in (1 - 1e-9, 1.0, 1 + 1e-9)])
    x = np.concatenate([-np.logspace(-8, 1, 6000), np.logspace(-8, 0.5, 3000), near, -near])
    out = np.zeros_like(x)
    L = capi.lib()
    rc = L.pn_selftest_phi1_f64(len(x), x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    exact = np.expm1(x) / x
    rel = np.abs(out - exact) / np.abs(exact)
    tol = np.where(np.abs(x) <= 2e-4, np.abs(x) ** 3 / 24 * 1.01 + 1e-15, 6e-15)
    assert np.all(rel <= tol), float(np.max(rel / tol))
