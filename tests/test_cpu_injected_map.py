"""The fp32 sampler's integer bin map for injected float64 uniforms.

``inj_bin_exact`` in csrc/vf_vegas_f32.cuh computes the reference's bin
``trunc(fl(50 * fl(1 - u)))`` (vflow.py:117, :67) from the exact value
50 (1 - u) in integer arithmetic and hands the cases it cannot decide (u outside
[2^-12, 1), or 50 (1 - u) within 2^-32 of an integer) back to the float64
operations.  This restates it in Python integers and checks the claim against
NumPy's float64 arithmetic on random, tiny and adversarial uniforms (values a
few ulps around every bin edge 1 - k/50)."""

import numpy as np

M64 = (1 << 64) - 1


def inj_bin_exact(u):
    """Python restatement of the device function: the bin, or None (float64 case)."""
    bits = int(np.float64(u).view(np.uint64))
    sh = (bits >> 52) - 1011  # includes the sign bit: negative u gives a large value
    if not 0 <= sh <= 11:
        return None
    mant = (bits & ((1 << 52) - 1)) | (1 << 52)
    v = (-(mant << sh)) & M64
    prod = v * 50  # 70-bit exact product: integer part above bit 64
    top = (prod >> 32) & 0xFFFFFFFF  # the fraction's top 32 bits
    if top == 0 or top == 0xFFFFFFFF:
        return None
    return prod >> 64


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


def test_out_of_range_goes_to_float64():
    for u in (-0.1, 1.0, 1.5, float("nan"), float("inf"), 2.0 ** -13):
        assert inj_bin_exact(u) is None
