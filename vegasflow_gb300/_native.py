"""ctypes binding of libvegasgb.so (the C-ABI declared in include/vegasflow_gb300.h).

The library is loaded lazily, from the in-tree build directory.  There is no
fallback: if the library is missing or no CUDA device is visible, every
compute entry point raises.
"""

from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libvegasgb.so")

VF_OK = 0
VF_ERR_ARG = 1
VF_ERR_LAUNCH = 2
VF_ERR_TIMEOUT = 3
VF_ERR_NONFINITE = 4
VF_ERR_JIT = 5
VF_ERR_CUDA = 6
VF_ERR_UNSUPPORTED = 7

VF_FLAG_INDEX_RANGE = 1
VF_FLAG_REFINE_OVERRUN = 2
VF_FLAG_NONFINITE = 4
VF_FLAG_TIMEOUT = 8
VF_FLAG_HISTORY_FULL = 16

VF_ALG_VEGAS = 0
VF_ALG_PLAIN = 1
VF_ALG_PLUS = 2
VF_ALG_BATCH = 3
VF_PREC_F64 = 0
VF_PREC_F32 = 1

VF_INT_NONE = 0
VF_INT_SYMGAUSS = 1
VF_INT_GAUSS = 2
VF_INT_BREIT_WIGNER = 3
VF_INT_PROD = 4
VF_INT_SUM = 5
VF_INT_JIT_BASE = 1000

VF_TUNE_F32_HIST_COPIES = 1
VF_TUNE_F32_THREADS = 2
VF_TUNE_F32_BLOCKS_PER_SM = 3

_P = ctypes.c_void_p
_I = ctypes.c_int
_LL = ctypes.c_longlong
_D = ctypes.c_double
_U64 = ctypes.c_ulonglong
_U32 = ctypes.c_uint

# name -> argument types (all return int status unless listed in _RESTYPE)
SIGNATURES = {
    "vf_version": [],
    "vf_last_error_string": [],
    "vf_device_info": [_P, _P, _P],
    "vf_sample_rows": [_I, _I, _I, _I, _I, _P],
    "vf_sample": [_I, _I, _P, _I, _LL, _LL, _D, _P, _P, _D, _P, _U64, _U32, _I, _P, _I, _I, _P, _I,
                  _P, _P, _P, _P, _P, _P],
    "vf_reduce_events": [_I, _P, _P, _P, _LL, _I, _I, _I, _I, _I, _P, _I, _P, _P],
    "vf_iteration_end": [_P, _I, _I, _I, _I, _D, _D, _P, _P, _P, _P, _P, _I, _P, _P],
    "vf_iteration_dev": [_I, _I, _P, _I, _LL, _D, _P, _P, _D, _U64, _P, _P, _I, _P, _I, _D, _P, _I, _P, _I, _P,
                         _P, _P],
    "vf_refine_grid": [_P, _P, _I, _D, _P, _P],
    "vf_consume_array_into_indices": [_P, _P, _LL, _I, _P, _P, _P],
    "vf_issue_probe": [_P, _I, _I, _P, _P],
    "vf_widemul_probe": [_P, _I, _I, _P, _P],
    "vf_vegas_iteration_static": [_I, _P, _I, _LL, _U64, _U32, _I, _P, _I, _P, _P, _P],
    "vf_philox_uniforms": [_U64, _U32, _U32, _LL, _LL, _I, _P, _P],
    "vf_plus_rows": [_I, _I, _I, _P],
    "vf_plus_sample": [_I, _P, _I, _I, _I, _P, _P, _D, _P, _P, _D, _P, _U64, _U32, _I, _P, _I, _P, _P,
                       _P, _I, _P, _P, _P, _P, _P],
    "vf_plus_reduce_events": [_I, _P, _P, _P, _P, _P, _I, _I, _I, _P, _P, _P, _I, _P],
    "vf_plus_iteration_end": [_P, _P, _P, _P, _I, _I, _I, _D, _P, _I, _I, _I, _D, _D, _P, _P, _P, _P,
                              _P, _I, _P, _P],
    "vf_plus_iteration_dev": [_I, _P, _I, _I, _I, _P, _P, _D, _P, _P, _D, _U64, _P, _P, _I, _P, _I, _I, _I, _D,
                              _D, _D, _P, _P, _P, _I, _P, _I, _P, _P, _P],
    "vf_batch_blocks": [_I, _P, _P],
    "vf_batch_sample": [_P, _P, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P, _U64, _P, _I, _P],
    "vf_batch_sample_jit": [_I, _P, _P, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P, _U64, _P, _I, _P],
    "vf_batch_iteration_end": [_P, _P, _P, _I, _P, _P, _P, _P, _P, _I, _P, _P, _P, _P, _P, _P],
    "vf_jit_integrand": [ctypes.c_char_p, ctypes.c_char_p, _I, _I, _I, _P],
    "vf_jit_check": [ctypes.c_char_p, ctypes.c_char_p, _I, _I, _I, ctypes.c_char_p, _I],
    "vf_preload": [],
    "vf_wait_selftest": [_I, _P, _P],
    "vf_tune_set": [_I, _I],
    "vf_tune_get": [_I, _P],
}
_RESTYPE = {"vf_last_error_string": ctypes.c_char_p}

_lock = threading.Lock()
_lib = None


class VegasGB300Error(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code, message):
        super().__init__(f"[vf error {code}] {message}")
        self.code = code


def load(path=LIB_PATH):
    """Load (once) and return the ctypes handle; raises if the library is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(
                f"libvegasgb.so not found at {path}: build it with `python -m vegasflow_gb300.build` "
                "(vegasflow_gb300 has no CPU fallback)")
        # make sure torch's CUDA runtime is resident first (one runtime per process)
        import torch  # noqa: F401
        lib = ctypes.CDLL(path)
        for name, argtypes in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = _RESTYPE.get(name, ctypes.c_int)
        _lib = lib
        return lib


def check(rc, what=""):
    if rc != VF_OK:
        msg = load().vf_last_error_string()
        raise VegasGB300Error(rc, (msg.decode() if msg else "") or what)


def call(name, *args):
    """Call an entry point and raise on a non-zero status."""
    rc = getattr(load(), name)(*args)
    check(rc, name)


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    """cudaStream_t of ``stream`` (default: the current stream of the current device)."""
    import torch
    if stream is not None:
        return ctypes.c_void_p(stream.cuda_stream)
    raw = getattr(torch._C, "_cuda_getCurrentRawStream", None)
    if raw is not None:  # the same handle without torch.cuda.current_stream()'s Python-side checks
        return ctypes.c_void_p(raw(torch._C._cuda_getDevice()))
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
