"""The NumPy stand-in for TensorFlow (``tests/golden/tfshim.py``) through which
the golden fixtures run the reference's own modules, checked op by op against
TensorFlow's documented semantics on the kinds of input the reference gives
them.  Where the documentation does not pin the behaviour (the maximum of a NaN
and a number), the test shows that no fixture reaches that case, so that no
golden value depends on the shim's choice there."""

import os
import sys

import numpy as np
import pytest

import oracle
from conftest import raw_blocks, replay_source

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import tfshim as tf  # noqa: E402


def _ulps32(a, b):
    a = np.asarray(a, dtype=np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, dtype=np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


def test_cast_float_to_int_truncates_toward_zero():
    """tf.cast: a float cast to an integer type drops the fraction (configflow.py:105,
    the bin index ``int_me(xn)`` of vflow.py:67 and ``int_me(new_n_ev)`` of vflowplus.py:162)."""
    x = np.array([-1.7, -0.5, 0.0, 0.5, 1.7, 49.999999, 2.0 ** 30 + 0.5])
    got = np.asarray(tf.cast(x, tf.int32))
    assert got.dtype == np.int32
    np.testing.assert_array_equal(got, [-1, 0, 0, 0, 1, 49, 2 ** 30])
    # float64 -> float32 rounds to nearest
    y = np.array([1.0 + 2.0 ** -24 + 2.0 ** -40, 1.0 / 3.0])
    np.testing.assert_array_equal(np.asarray(tf.cast(y, tf.float32)), y.astype(np.float32))


def test_gather_batch_dims_1_is_per_row():
    """tf.gather(params, indices, batch_dims=1): out[i, j] = params[i, indices[i, j]]
    (vflow.py:70-71: the bin edges of every event, per dimension)."""
    rng = np.random.default_rng(0)
    params = rng.random((3, 51))
    indices = rng.integers(0, 51, (3, 200)).astype(np.int32)
    got = np.asarray(tf.gather(params, indices, batch_dims=1))
    want = np.array([[params[i, indices[i, j]] for j in range(200)] for i in range(3)])
    np.testing.assert_array_equal(got, want)


def test_gather_rows():
    """tf.gather(params, indices) picks rows along axis 0 (vflowplus.py:68-69: the
    hypercube of every event)."""
    params = np.arange(12, dtype=np.int32).reshape(6, 2)
    idx = np.array([5, 0, 0, 3], dtype=np.int32)
    np.testing.assert_array_equal(np.asarray(tf.gather(params, idx)), params[idx])


def test_reduce_prod_and_sum():
    """tf.reduce_prod(x, axis=0) multiplies the rows (vflow.py:78: the weight over the
    dimensions); tf.reduce_sum over an axis or everything; dtypes are kept."""
    rng = np.random.default_rng(1)
    x = rng.random((4, 7))
    got = np.asarray(tf.reduce_prod(x, axis=0))
    assert got.dtype == np.float64 and got.shape == (7,)
    np.testing.assert_array_equal(got, ((x[0] * x[1]) * x[2]) * x[3])
    assert np.asarray(tf.reduce_prod(np.array([2.0, 3.0, 4.0]))) == 24.0
    np.testing.assert_allclose(np.asarray(tf.reduce_sum(x, axis=1)), x.sum(axis=1), rtol=1e-15)
    x32 = x.astype(np.float32)
    assert np.asarray(tf.reduce_prod(x32, axis=0)).dtype == np.float32


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_pow_keeps_dtype_and_is_faithful(dtype):
    """tf.pow(x, y) with a Python float exponent converts the exponent to x's dtype
    and computes in it (vflow.py:165 ``aux ** ALPHA``; vflowplus.py:157
    ``var ** (BETA / 2)``): the result keeps the dtype and is within one unit in
    the last place of the exact power of the converted exponent."""
    rng = np.random.default_rng(2)
    x = (rng.random(5000) * 10.0 ** rng.integers(-6, 3, 5000)).astype(dtype)
    for y in (1.5, 0.375, 1.0 / 3.0):
        got = np.asarray(tf.pow(x, y))
        assert got.dtype == dtype
        exact = np.power(x.astype(np.longdouble), np.longdouble(dtype(y)))
        if dtype == np.float32:
            assert _ulps32(got, exact.astype(np.float32)).max() <= 1
        else:
            np.testing.assert_allclose(got, exact.astype(np.float64), rtol=2.3e-16, atol=0)
    # two Python scalars: float32, as TensorFlow converts a bare Python float
    # (vflowplus.py:115, ``pow(neval_eff / 2, 1 / n_dim)``)
    assert np.asarray(tf.math.pow(2500.0, 1.0 / 3.0)).dtype == np.float32


def test_elementwise_and_constructors():
    """tf.math.floor / log, tf.sqrt, tf.square, tf.fill (dtype of the value), tf.pad
    with a constant (vflow.py:152-158), tf.range of integers."""
    x = np.array([-1.5, -0.0, 0.25, 2.0, 7.999999])
    np.testing.assert_array_equal(np.asarray(tf.math.floor(x)), np.floor(x))
    pos = np.array([1e-30, 0.5, 1.0, 3.0])
    np.testing.assert_array_equal(np.asarray(tf.math.log(pos)), np.log(pos))
    np.testing.assert_array_equal(np.asarray(tf.sqrt(pos)), np.sqrt(pos))
    np.testing.assert_array_equal(np.asarray(tf.square(x)), x * x)
    f = np.asarray(tf.fill([48], np.float64(3.0)))
    assert f.dtype == np.float64 and f.shape == (48,) and np.all(f == 3.0)
    p = np.asarray(tf.pad(f, np.array([[1, 1]], dtype=np.int32), constant_values=2.0))
    assert p.shape == (50,) and p[0] == 2.0 and p[-1] == 2.0 and np.all(p[1:-1] == 3.0)
    r = np.asarray(tf.range(np.int32(5)))
    assert r.dtype == np.int32
    np.testing.assert_array_equal(r, np.arange(5))


def test_segment_sum_with_empty_segments():
    """tf.math.segment_sum (vflowplus.py:213-214): one sum per id 0..max(id), an id
    with no entries sums to 0."""
    data = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    ids = np.array([0, 0, 2, 2, 4], dtype=np.int32)
    got = np.asarray(tf.math.segment_sum(data, ids))
    np.testing.assert_array_equal(got, [3.0, 0.0, 7.0, 0.0, 5.0])
    assert got.dtype == np.float64


def test_maximum_on_numbers():
    """tf.maximum on finite numbers and infinities is the elementwise maximum
    (plain.py:42, vflow.py:159, :438, vflowplus.py:158, :230)."""
    a = np.array([-1.0, 0.0, 1e-31, np.inf, -np.inf, 5.0])
    b = np.array([0.0, -0.0, 1e-30, 1.0, 2.0, 5.0])
    np.testing.assert_array_equal(np.asarray(tf.maximum(a, b)), np.maximum(a, b))
    # a Python scalar on either side
    np.testing.assert_array_equal(np.asarray(tf.maximum(a, 1e-30)), np.maximum(a, 1e-30))


def test_no_fixture_takes_the_maximum_of_a_nan(golden):
    """TensorFlow's documentation does not fix tf.maximum(number, NaN); the shim
    returns the number.  Of the reference's tf.maximum calls, only the VEGAS+
    redistribution (vflowplus.py:157-160) can meet a NaN: the power 0.375 of a
    hypercube variance that rounding made negative.  Replaying the adaptive
    golden case, every variance that reaches it is >= 0 (and every other
    maximum's operands are finite), so no golden value depends on that choice."""
    source = replay_source(raw_blocks(golden, "plus3_adaptive"), oracle.tech_cut_affine)
    seen = []
    real = oracle.redistribute_samples

    def spy(arr_var, min_neval, init_calls):
        seen.append(np.array(arr_var))
        return real(arr_var, min_neval, init_calls)

    inst = oracle.OraclePlus(3, 4000, adaptive=True)
    oracle.vegas_oracle.redistribute_samples = spy
    try:
        for _ in range(3):
            inst.iteration(source, lambda x: oracle.integrand_symgauss(x, 0.1))
            assert np.all(np.isfinite(inst.last["arr_res2"]))
    finally:
        oracle.vegas_oracle.redistribute_samples = real
    assert len(seen) == 3
    for v in seen:
        assert np.all(np.isfinite(v)) and np.all(v >= 0.0)
