"""Truncation bounds of the FP64 exponential factor's series ranges (the device's phi1 in
pn_device.cuh): sum_{k<=K} c^k/(k+1)! with K = 6, 8, 10, 14 below |c| = 0.03, 0.1, 0.3, 0.7."""
import math

import numpy as np

RANGES = [(0.03, 6), (0.1, 8), (0.3, 10), (0.7, 14)]


def series(c, K):
    t = 1.0 / math.factorial(K + 1)
    for k in range(K - 1, -1, -1):
        t = t * c + 1.0 / math.factorial(k + 1)
    return t


def test_series_ranges_meet_their_truncation_bounds():
    lo = 2e-4
    for hi, K in RANGES:
        for c in np.concatenate([np.linspace(lo, hi, 200), -np.linspace(lo, hi, 200)]):
            exact = math.expm1(c) / c
            rel = abs(series(c, K) - exact) / abs(exact)
            # 4.3e-15 is the truncation at 0.3 with K = 10; the others stay near 5e-16
            assert rel < (5e-15 if K == 10 else 1e-15), (c, K, rel)
        lo = hi


def test_one_term_fewer_would_miss_the_bound():
    """Each range uses the fewest terms that keep its truncation near the FP64 rounding level."""
    for hi, K in RANGES:
        c = -hi
        exact = math.expm1(c) / c
        assert abs(series(c, K - 1) - exact) / exact > 1e-15
