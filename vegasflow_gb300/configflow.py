"""Constants, environment flags, dtypes and casts (vegasflow configflow.py).

Same names and meanings as the reference (configflow.py:13-116): ``BINS_MAX``,
``ALPHA``, ``BETA``, ``TECH_CUT``, ``MAX_EVENTS_LIMIT``, ``MAX_NEVAL_HCUBE``,
``DEFAULT_ACTIVE_DEVICES``; the ``VEGASFLOW_LOG_LEVEL`` / ``VEGASFLOW_FLOAT`` /
``VEGASFLOW_INT`` environment variables; ``DTYPE`` / ``DTYPEINT`` (torch dtypes
here); ``float_me`` / ``int_me`` / ``run_eager``.

``VEGASFLOW_FLOAT=32`` selects the fused fp32 form of the samplers (fp32
sampling and evaluation, compensated sums, float64 across blocks and
iterations) as the integrators' default precision.
"""

from __future__ import annotations

import logging
import os

import numpy as np
import torch

BINS_MAX = 50
ALPHA = 1.5
BETA = 0.75  # VEGAS+
TECH_CUT = 1e-8

MAX_EVENTS_LIMIT = int(1e6)
MAX_NEVAL_HCUBE = int(1e4)

DEFAULT_ACTIVE_DEVICES = ["GPU"]

LOG_DICT = {"0": logging.ERROR, "1": logging.WARNING, "2": logging.INFO, "3": logging.DEBUG}

_log_level_idx = os.environ.get("VEGASFLOW_LOG_LEVEL")
_float_env = os.environ.get("VEGASFLOW_FLOAT", "64")
_int_env = os.environ.get("VEGASFLOW_INT", "32")

if _log_level_idx not in LOG_DICT:
    _log_level_idx = None
_log_level = LOG_DICT["2"] if _log_level_idx is None else LOG_DICT[_log_level_idx]

logger = logging.getLogger("vegasflow")
logger.setLevel(_log_level)
if not any(getattr(h, "_vegasflow_gb300", False) for h in logger.handlers):
    _console_handler = logging.StreamHandler()
    _console_handler.setLevel(_log_level)
    _console_handler.setFormatter(logging.Formatter("[%(levelname)s] (%(name)s) %(message)s"))
    _console_handler._vegasflow_gb300 = True
    logger.addHandler(_console_handler)

if _float_env == "64":
    DTYPE = torch.float64
elif _float_env == "32":
    DTYPE = torch.float32
else:
    DTYPE = torch.float64
    logger.warning(f"VEGASFLOW_FLOAT={_float_env} not understood, defaulting to 64 bits")

if _int_env == "64":
    DTYPEINT = torch.int64
elif _int_env == "32":
    DTYPEINT = torch.int32
else:
    DTYPEINT = torch.int64
    logger.warning(f"VEGASFLOW_INT={_int_env} not understood, defaulting to 64 bits")

FMAX = float(np.finfo(np.float64).max)

# the precision mode the integrators use unless told otherwise
DEFAULT_PRECISION = "fp64" if DTYPE == torch.float64 else "fp32"


def run_eager(flag=True):
    """Kept for API compatibility: there is no graph compiler to bypass here
    (the hot path is ahead-of-time CUDA), so this only records the flag."""
    global _RUN_EAGER
    _RUN_EAGER = bool(flag)


_RUN_EAGER = False


def int_me(i):
    """Cast the input to ``DTYPEINT`` (a torch tensor on the input's device)."""
    if isinstance(i, torch.Tensor):
        return i.to(DTYPEINT)
    return torch.as_tensor(np.asarray(i), dtype=DTYPEINT)


def float_me(i):
    """Cast the input to ``DTYPE`` (a torch tensor on the input's device)."""
    if isinstance(i, torch.Tensor):
        return i.to(DTYPE)
    return torch.as_tensor(np.asarray(i, dtype=np.float64), dtype=DTYPE)


ione = int_me(1)
izero = int_me(0)
fone = float_me(1)
fzero = float_me(0)
