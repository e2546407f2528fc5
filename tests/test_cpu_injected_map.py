"""The fp32 sampler's integer bin map for injected float64 uniforms.

``inj_bin_exact`` in csrc/vf_vegas_f32.cuh computes the reference's bin
``trunc(fl(50 * fl(1 - u)))`` (vflow.py:117, :67) from 50 (1 - u) 2^32 =
P + c, P = 50 (2^32 - 1 - high word of u 2^64), c in [0, 50], in integer
arithmetic and hands the cases it cannot decide (u outside [2^-12, 1), or the
low word of P within 52 of an integer boundary) back to the float64
operations.  This restates it in Python integers and checks the claim against
NumPy's float64 arithmetic on random, tiny and adversarial uniforms (values a
few ulps around every bin edge 1 - k/50), and the fraction it returns against
the exact one."""

import numpy as np

M64 = (1 << 64) - 1


def inj_bin_exact(u, with_m=False):
    """Python restatement of the device function: the bin (and m), or None (float64 case)."""
    bits = int(np.float64(u).view(np.uint64))
    sh = (bits >> 52) - 1011  # includes the sign bit: negative u gives a large value
    if not 0 <= sh <= 11:
        return None
    mant = (bits & ((1 << 52) - 1)) | (1 << 52)
    h = ((mant << sh) >> 32) & 0xFFFFFFFF  # the high word of U = u 2^64
    p = (~h & 0xFFFFFFFF) * 50
    f = p & 0xFFFFFFFF
    if not 1 <= f <= (1 << 32) - 52:
        return None
    if with_m:
        return p >> 32, 1.0 + (f >> 9) / 2.0 ** 23
    return p >> 32


def _adversarial():
    out = []
    for k in range(51):
        x = y = 1.0 - k / 50.0
        out.append(x)
        for _ in range(64):
            x = np.nextafter(x, 2.0)
            y = np.nextafter(y, -1.0)
            out += [x, y]
    return np.array(out)


def test_integer_map_matches_float64():
    rng = np.random.default_rng(0)
    us = np.concatenate([rng.random(200_000), 10.0 ** rng.uniform(-12, 0, 20_000), _adversarial(),
                         np.array([0.0, 1e-8, 1.0 - 1e-8, 0.5, 0.25, np.nextafter(1.0, 0.0)])])
    want = (50.0 * (1.0 - us)).astype(np.int64)
    fast = 0
    for u, w in zip(us, want):
        got = inj_bin_exact(u)
        if got is not None:
            fast += 1
            assert got == w, (u, got, w)
    assert fast > 0.9 * us.size  # the float64 fallback stays rare


def test_fraction_within_one_step_of_exact():
    """m = 1 + the top 23 bits of P's low word: below 1 + the exact fraction of
    50 (1 - u) by less than 2^-23 (the truncation) + 51 2^-32 (the dropped c)."""
    from fractions import Fraction

    rng = np.random.default_rng(1)
    for u in np.concatenate([rng.random(20_000), _adversarial()[::7]]):
        r = inj_bin_exact(u, with_m=True)
        if r is None:
            continue
        ind, m = r
        y = 50 * (1 - Fraction(float(u)))
        assert ind == int(y)
        gap = (1 + (y - int(y))) - Fraction(m)
        assert 0 <= gap < Fraction(1, 1 << 23) + Fraction(51, 1 << 32), (u, float(gap))


def test_out_of_range_goes_to_float64():
    for u in (-0.1, 1.0, 1.5, float("nan"), float("inf"), 2.0 ** -13):
        assert inj_bin_exact(u) is None
