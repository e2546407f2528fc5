"""The fp32 VEGAS+ sampler's integer stratified map (csrc/vf_plus_f32.cuh):
Q = 50 (p 2^32 + w) + 25, A = Q >> 32, bin = A div n_strat through a float32
reciprocal corrected by one step, fraction from the remainder.  Restated here
with NumPy float32 and checked against exact integer and rational arithmetic
for n_strat up to the reference's 10^4 cap (vflowplus.py:115-123)."""

from fractions import Fraction

import numpy as np


def device_div(A, n):
    """A div n as the kernel computes it (A < 50 n < 2^24)."""
    inv = np.float32(1.0) / np.float32(n)
    i = np.uint32(np.float32(A) * inv)
    if i * n > A:
        i -= 1
    if (i + 1) * n <= A:
        i += 1
    return int(i)


def test_division_exact_for_all_strata_counts():
    rng = np.random.default_rng(0)
    for n in list(range(1, 200)) + list(rng.integers(200, 10_001, 300)):
        n = int(n)
        A = np.concatenate([np.arange(min(50 * n, 2000)), rng.integers(0, 50 * n, 2000),
                            np.arange(n - 1, 50 * n, n), np.arange(0, 50 * n, n)])
        for a in A:
            a = int(a)
            assert device_div(a, n) == a // n, (a, n)


def test_bin_and_fraction_are_the_stratified_coordinate():
    """bin = floor(xn) and 1 + fraction ~ 1 + frac(xn) for xn = (p + u) 50 / n,
    u = (w + 1/2) / 2^32, within float32 rounding."""
    rng = np.random.default_rng(1)
    for _ in range(3000):
        n = int(rng.integers(1, 10_001))
        p = int(rng.integers(0, n))
        w = int(rng.integers(0, 2 ** 32))
        Q = 50 * ((p << 32) | w) + 25
        A, R = Q >> 32, Q & 0xFFFFFFFF
        i = device_div(A, n)
        r = A - i * n
        m = np.float32(1.0) + (np.float32(R) * np.float32(2.3283064e-10) + np.float32(r)) * (np.float32(1.0) / np.float32(n))
        m = min(m, np.float32(1.99999988))
        xn = (Fraction(p) + Fraction(2 * w + 1, 2 ** 33)) * 50 / n
        assert i == int(xn) and 0 <= i < 50
        assert abs(float(m) - 1.0 - float(xn - int(xn))) < 4e-7
