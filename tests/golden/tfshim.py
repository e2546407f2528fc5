"""A NumPy-backed stand-in for the TensorFlow calls made by vegasflow 1.4.0.

TensorFlow is not installed here, so ``make_golden.py`` installs this module as
``tensorflow`` before importing the reference package.  The reference's Python
modules (``src/vegasflow/*.py``) then run unmodified, eagerly, with every tensor
a NumPy array.  Only the operations those modules call are provided, each with
TensorFlow's semantics for the dtypes involved:

* ``tf.cast`` float->int truncates toward zero; Python-float operands of
  ``tf.math.pow`` become float32 tensors (TensorFlow's default float dtype).
* ``tf.random.uniform(shape, minval, maxval)`` returns ``u * (maxval - minval) +
  minval`` where ``u`` comes from an *injected* source (see ``set_uniform_source``),
  so the reference's sampling can be replayed on known uniforms.
* ``tf.maximum(a, NaN)`` returns ``a`` (Eigen's std::max ordering), via ``fmax``.
* Reductions use NumPy's summation order (TensorFlow's own order is an Eigen
  implementation detail); results differ from a TensorFlow run only by rounding.

Test infrastructure only: used by ``make_golden.py`` in the development
container, never by the product package or on the GPU host.
"""

from __future__ import annotations

import builtins
import contextlib
import logging
import types

import numpy as np

__version__ = "2.99.0-numpy-shim"


class Tensor(np.ndarray):
    """ndarray that keeps 0-d results as arrays and offers ``numpy``/``assign``."""

    def __array_wrap__(self, obj, context=None, return_scalar=False):
        if isinstance(obj, np.ndarray):
            return obj.view(Tensor)
        return obj

    def numpy(self):
        return np.asarray(self).copy() if self.ndim else np.asarray(self)[()]

    def assign(self, value):
        self[...] = np.asarray(value)
        return self

    def __hash__(self):
        return id(self)

    # TensorFlow tensors are immutable: ``a += b`` rebinds ``a`` to a new tensor.
    def __iadd__(self, other):
        return np.add(self, other)

    def __isub__(self, other):
        return np.subtract(self, other)

    def __imul__(self, other):
        return np.multiply(self, other)

    def __itruediv__(self, other):
        return np.true_divide(self, other)


def _t(x, dtype=None):
    arr = np.asarray(x, dtype=dtype)
    return arr.view(Tensor)


class DType:
    def __init__(self, name, np_dtype):
        self.name = name
        self.as_numpy_dtype = np_dtype

    def __repr__(self):
        return f"tf.{self.name}"


float64 = DType("float64", np.float64)
float32 = DType("float32", np.float32)
int64 = DType("int64", np.int64)
int32 = DType("int32", np.int32)
bool = DType("bool", np.bool_)  # noqa: A001


def _np_dtype(dtype):
    if dtype is None:
        return None
    if isinstance(dtype, DType):
        return dtype.as_numpy_dtype
    return dtype


def _infer(x):
    """TensorFlow's dtype inference for Python scalars/lists: float -> float32,
    int -> int32; NumPy arrays keep their dtype."""
    if isinstance(x, np.ndarray):
        return x
    arr = np.asarray(x)
    if arr.dtype == np.float64 and not isinstance(x, np.floating):
        return arr.astype(np.float32)
    if arr.dtype == np.int64 and not isinstance(x, np.integer):
        return arr.astype(np.int32)
    return arr


class TensorSpec:
    def __init__(self, shape=None, dtype=None, name=None):
        self.shape = shape
        self.dtype = dtype

    def __repr__(self):
        return f"TensorSpec({self.shape}, {self.dtype})"


def function(func=None, input_signature=None, **kwargs):
    if func is None:
        return lambda f: f
    return func


def constant(value, dtype=None):
    return _t(value, _np_dtype(dtype))


def cast(x, dtype):
    return _t(np.asarray(x).astype(_np_dtype(dtype)))


def convert_to_tensor(value, dtype=None):
    return _t(value, _np_dtype(dtype))


def Variable(value, dtype=None):  # noqa: N802
    return _t(np.array(value, dtype=_np_dtype(dtype), copy=True))


def reshape(x, shape):
    return _t(np.reshape(np.asarray(x), shape))


def transpose(x):
    return _t(np.asarray(x).T)


def gather(params, indices, batch_dims=0, axis=None):
    params = np.asarray(params)
    indices = np.asarray(indices)
    if batch_dims == 1:
        return _t(np.take_along_axis(params, indices, axis=1))
    return _t(params[indices])


def reduce_sum(x, axis=None):
    if isinstance(x, list):
        x = np.array([np.asarray(v) for v in x])
    return _t(np.sum(np.asarray(x), axis=axis))


def reduce_prod(x, axis=None):
    x = np.asarray(x)
    if axis == 0 and x.ndim >= 1 and x.shape[0] > 0:
        acc = x[0].copy()
        for i in range(1, x.shape[0]):
            acc = acc * x[i]
        return _t(acc)
    return _t(np.prod(x, axis=axis))


def square(x):
    x = np.asarray(x)
    return _t(x * x)


def sqrt(x):
    return _t(np.sqrt(np.asarray(x)))


def exp(x):
    return _t(np.exp(np.asarray(x)))


def _pair(x, y):
    """The operands of a binary op: a Python scalar beside a tensor takes the
    tensor's dtype (converted once, not through float32); two Python scalars
    follow ``_infer``."""
    xt, yt = isinstance(x, np.ndarray), isinstance(y, np.ndarray)
    if xt and not yt:
        return x, np.asarray(y, dtype=x.dtype)
    if yt and not xt:
        return np.asarray(x, dtype=y.dtype), y
    return _infer(x), _infer(y)


def maximum(x, y):
    x, y = _pair(x, y)
    return _t(np.fmax(x, y))


def pow(x, y):  # noqa: A001
    x, y = _pair(x, y)
    with np.errstate(invalid="ignore"):
        return _t(np.power(x, y))


def fill(dims, value):
    value = _infer(value)
    return _t(np.full(dims, value, dtype=value.dtype))


def pad(x, paddings, constant_values=0):
    pads = [tuple(int(v) for v in p) for p in np.asarray(paddings)]
    return _t(np.pad(np.asarray(x), pads, constant_values=constant_values))


def range(start, limit=None, delta=1, dtype=None):  # noqa: A001
    start = np.asarray(start)
    if limit is None:
        limit, start = start, np.zeros((), dtype=start.dtype)
    out = np.arange(start, limit, delta)
    if dtype is not None:
        out = out.astype(_np_dtype(dtype))
    elif np.asarray(limit).dtype.kind == "i" and start.dtype.kind == "i":
        out = out.astype(np.asarray(limit).dtype)
    return _t(out)


def repeat(x, repeats):
    return _t(np.repeat(np.asarray(x), np.asarray(repeats)))


def shape(x, out_type=None):
    return _t(np.asarray(np.asarray(x).shape, dtype=_np_dtype(out_type) or np.int32))


def stack(values, axis=0):
    return _t(np.stack([np.asarray(v) for v in values], axis=axis))


def concat(values, axis=0):
    return _t(np.concatenate([np.asarray(v) for v in values], axis=axis))


def equal(x, y):
    return _t(np.equal(np.asarray(x), np.asarray(y)))


def where(cond, x=None, y=None):
    if x is None:
        return _t(np.argwhere(np.asarray(cond)))
    return _t(np.where(np.asarray(cond), np.asarray(x), np.asarray(y)))


def zeros_like(x, dtype=None):
    return _t(np.zeros_like(np.asarray(x), dtype=_np_dtype(dtype)))


def while_loop(cond, body, loop_vars, **kwargs):
    loop_vars = tuple(loop_vars)
    while builtins.bool(cond(*loop_vars)):
        loop_vars = tuple(body(*loop_vars))
    return loop_vars


def device(name):
    return contextlib.nullcontext()


def get_logger():
    return logging.getLogger("tensorflow")


# -- tf.math ------------------------------------------------------------------
def _floor(x):
    return _t(np.floor(_infer(x)))


def _log(x):
    return _t(np.log(np.asarray(x)))


def _segment_sum(data, segment_ids):
    ids = np.asarray(segment_ids)
    n_seg = int(ids.max()) + 1 if ids.size else 0
    return _t(np.bincount(ids, weights=np.asarray(data, dtype=np.float64), minlength=n_seg))


math = types.SimpleNamespace(
    floor=_floor, pow=pow, log=_log, segment_sum=_segment_sum, exp=exp,
    logical_and=lambda a, b: _t(np.logical_and(a, b)),
    logical_or=lambda a, b: _t(np.logical_or(a, b)),
    reduce_all=lambda x, axis=None: _t(np.all(np.asarray(x), axis=axis)),
    reduce_any=lambda x, axis=None: _t(np.any(np.asarray(x), axis=axis)),
)


# -- tf.random: injected uniform source ---------------------------------------
_state = {"source": None, "aux": np.random.default_rng(12345)}


def set_uniform_source(fn):
    """``fn(shape) -> float64 U[0,1) array`` feeds the reference's sampling draws
    (the ones made with ``minval=TECH_CUT``); other draws (the compile-time shape
    check) come from a private generator."""
    _state["source"] = fn


def _uniform(shape, minval=0, maxval=None, dtype=float32, seed=None):
    shape = tuple(int(s) for s in np.atleast_1d(np.asarray(shape, dtype=np.int64)))
    npd = _np_dtype(dtype)
    if minval != 0 and _state["source"] is not None:
        raw = np.asarray(_state["source"](shape), dtype=np.float64)
    else:
        raw = _state["aux"].random(shape)
    raw = raw.astype(npd)
    if minval == 0 and (maxval is None or maxval == 1):
        return _t(raw)
    lo = np.asarray(minval, dtype=npd)
    hi = np.asarray(1 if maxval is None else maxval, dtype=npd)
    return _t(raw * (hi - lo) + lo)


random = types.SimpleNamespace(uniform=_uniform, set_seed=lambda s: None)


# -- tf.config / tf.autograph ---------------------------------------------------
def _list_logical_devices(device_type=None):
    return [types.SimpleNamespace(name="/device:CPU:0", device_type="CPU")]


config = types.SimpleNamespace(
    run_functions_eagerly=lambda flag: None,
    experimental_run_functions_eagerly=lambda flag: None,
    experimental=types.SimpleNamespace(list_logical_devices=_list_logical_devices),
)
autograph = types.SimpleNamespace(
    experimental=types.SimpleNamespace(Feature=types.SimpleNamespace(ALL="ALL"))
)
