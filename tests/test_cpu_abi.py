"""CPU checks of the C-ABI library: it builds, loads without a GPU, and exports
every entry point the public header declares (no compute calls here)."""

import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "vegasflow_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(vf_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    from vegasflow_gb300.build import LIB, build

    if not os.path.exists(LIB):
        build()
    return ctypes.CDLL(LIB)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for name in ("vf_sample", "vf_iteration_end", "vf_refine_grid", "vf_reduce_events",
                 "vf_consume_array_into_indices", "vf_last_error_string"):
        assert name in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    from vegasflow_gb300 import _native

    assert set(declared_symbols()) <= set(_native.SIGNATURES), \
        set(declared_symbols()) - set(_native.SIGNATURES)


def test_version_and_error_string(lib):
    lib.vf_version.restype = ctypes.c_int
    assert lib.vf_version() >= 1
    lib.vf_last_error_string.restype = ctypes.c_char_p
    assert isinstance(lib.vf_last_error_string(), bytes)


def test_constants_match_header():
    from vegasflow_gb300 import _native as nat

    text = open(HEADER).read()
    for name in ("VF_OK", "VF_ERR_ARG", "VF_ALG_VEGAS", "VF_ALG_PLAIN", "VF_PREC_F64", "VF_PREC_F32",
                 "VF_INT_NONE", "VF_INT_SYMGAUSS", "VF_INT_GAUSS", "VF_INT_BREIT_WIGNER",
                 "VF_INT_PROD", "VF_INT_SUM", "VF_FLAG_INDEX_RANGE", "VF_FLAG_REFINE_OVERRUN",
                 "VF_FLAG_NONFINITE", "VF_INT_JIT_BASE"):
        m = re.search(rf"#define\s+{name}\s+(\d+)", text)
        assert m, name
        assert getattr(nat, name) == int(m.group(1)), name


def test_binding_argument_counts_match_header():
    """Every ctypes signature has as many arguments as the C prototype."""
    from vegasflow_gb300 import _native

    text = open(HEADER).read()
    for m in re.finditer(r"^(?:int|const char\*)\s+(vf_\w+)\s*\((.*?)\);", text, re.M | re.S):
        name, params = m.group(1), " ".join(m.group(2).split())
        n = 0 if params in ("", "void") else params.count(",") + 1
        assert len(_native.SIGNATURES[name]) == n, (name, n, len(_native.SIGNATURES[name]))


def test_binding_argument_types_match_header():
    """Pointers bind as pointers, and each scalar with the ctypes type of its C type."""
    from vegasflow_gb300 import _native

    scalar = {"int": ctypes.c_int, "double": ctypes.c_double, "long long": ctypes.c_longlong,
              "unsigned long long": ctypes.c_ulonglong, "unsigned int": ctypes.c_uint}
    text = open(HEADER).read()
    for m in re.finditer(r"^(?:int|const char\*)\s+(vf_\w+)\s*\((.*?)\);", text, re.M | re.S):
        name, params = m.group(1), " ".join(m.group(2).split())
        if params in ("", "void"):
            continue
        for k, (param, bound) in enumerate(zip(params.split(","), _native.SIGNATURES[name])):
            param = param.strip()
            if "*" in param:
                assert bound in (ctypes.c_void_p, ctypes.c_char_p), (name, k, param)
            else:
                ctype = " ".join(t for t in param.split()[:-1] if t != "const")
                assert bound is scalar[ctype], (name, k, param, bound)
