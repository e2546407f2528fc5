"""The allocation-free VEGAS iteration, ``vf_vegas_iteration_static``.

Callers that cannot allocate device memory -- a plugin whose host framework
owns every device allocation, code that must not allocate while a stream is
captured, a fixed-budget deployment -- use this entry point: its scratch (the
per-block partial sums) lives in a fixed array inside the library, so they pass
only the grid, the integrand parameters and a 2-double output.

These tests call it through the C-ABI and compare two consecutive iterations
with the regular entry points (``vf_sample`` + ``vf_iteration_end`` with a
caller-owned scratch buffer) on the same seed: result, sigma and the refined
grid agree within the tolerances of the other parity tests (1e-10 relative in
float64; 2e-5 in the fp32 form, whose per-block sums depend on the block
count).  The file is collected last so that a failure here never hides another.
"""

import ctypes

import numpy as np
import pytest
import torch

from vegasflow_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("precision,rtol,grid_atol", [(nat.VF_PREC_F64, 1e-10, 1e-12),
                                                     (nat.VF_PREC_F32, 2e-5, 1e-5)])
def test_static_iteration_matches_regular_path(precision, rtol, grid_atol):
    lib = nat.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    n_dim, n_events, seed = 6, 300_000, 1234
    grid0 = np.linspace(0.0, 1.0, 51)[None, :].repeat(n_dim, 0)
    grid_static = torch.tensor(grid0, dtype=torch.float64, device=dev)
    grid_regular = grid_static.clone()
    params = torch.tensor([0.1, (1.0 / 0.1 / np.sqrt(np.pi)) ** n_dim], dtype=torch.float64, device=dev)
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    flags = torch.full((1,), -1, dtype=torch.int32, device=dev)
    stream = nat.stream_handle()

    rows = ctypes.c_int(0)
    assert lib.vf_sample_rows(nat.VF_ALG_VEGAS, precision, n_dim, nat.VF_INT_SYMGAUSS, 1,
                              ctypes.byref(rows)) == 0
    partials = torch.zeros(rows.value * (2 + 50 * n_dim), dtype=torch.float64, device=dev)
    history = torch.zeros((2, 2), dtype=torch.float64, device=dev)
    avg = torch.zeros(5, dtype=torch.float64, device=dev)

    for call in (0, 1):
        rc = lib.vf_vegas_iteration_static(precision, _p(grid_static), n_dim, n_events, seed, call,
                                           nat.VF_INT_SYMGAUSS, _p(params), 1, _p(out), _p(flags), stream)
        assert rc == nat.VF_OK, lib.vf_last_error_string()
        got = out.cpu().numpy().copy()
        assert int(flags.item()) == 0  # written by every call, nothing went wrong

        nat.check(lib.vf_sample(nat.VF_ALG_VEGAS, precision, _p(grid_regular), n_dim, n_events, 0,
                                1.0 / n_events, None, None, 1.0, None, seed, call, nat.VF_INT_SYMGAUSS,
                                _p(params), 1, 0, _p(partials), rows.value, None, None, None, None,
                                None, stream))
        nat.check(lib.vf_iteration_end(_p(partials), rows.value, n_dim, 1, 1, float(n_events), 1.5,
                                       _p(grid_regular), None, None, _p(history), _p(avg), call, None,
                                       stream))
        want = history[call].cpu().numpy()
        np.testing.assert_allclose(got, want, rtol=rtol)
        np.testing.assert_allclose(grid_static.cpu().numpy(), grid_regular.cpu().numpy(),
                                   rtol=0, atol=grid_atol)
        assert abs(got[0] - 1.0) < 6 * got[1] + 1e-3


def test_static_iteration_rejects_unsupported_sizes():
    lib = nat.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    grid = torch.zeros((17, 51), dtype=torch.float64, device=dev)
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    rc = lib.vf_vegas_iteration_static(nat.VF_PREC_F64, _p(grid), 17, 1000, 1, 0, nat.VF_INT_PROD, None,
                                       1, _p(out), None, nat.stream_handle())
    assert rc == nat.VF_ERR_UNSUPPORTED
    assert b"n_dim" in lib.vf_last_error_string()
    # train outside 0..2 is refused before anything reaches the stream
    grid4 = torch.tensor(np.linspace(0.0, 1.0, 51)[None, :].repeat(4, 0), device=dev)
    rc = lib.vf_vegas_iteration_static(nat.VF_PREC_F32, _p(grid4), 4, 1000, 1, 0, nat.VF_INT_PROD, None,
                                       3, _p(out), None, nat.stream_handle())
    assert rc == nat.VF_ERR_ARG
    assert b"train" in lib.vf_last_error_string()


@pytest.mark.parametrize("precision", [nat.VF_PREC_F64, nat.VF_PREC_F32])
def test_static_iteration_reports_device_flags(precision):
    """A non-finite sum reaches the caller through flags_out (an infinite
    normalisation makes every weight infinite), and the next clean call writes 0."""
    lib = nat.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    n_dim, n_events = 4, 100_000
    grid = torch.tensor(np.linspace(0.0, 1.0, 51)[None, :].repeat(n_dim, 0), device=dev)
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    flags = torch.zeros(1, dtype=torch.int32, device=dev)
    bad = torch.tensor([0.1, float("inf")], dtype=torch.float64, device=dev)
    rc = lib.vf_vegas_iteration_static(precision, _p(grid), n_dim, n_events, 5, 0, nat.VF_INT_SYMGAUSS,
                                       _p(bad), 0, _p(out), _p(flags), nat.stream_handle())
    assert rc == nat.VF_OK, lib.vf_last_error_string()
    assert int(flags.item()) & nat.VF_FLAG_NONFINITE
    good = torch.tensor([0.1, (1.0 / 0.1 / np.sqrt(np.pi)) ** n_dim], dtype=torch.float64, device=dev)
    rc = lib.vf_vegas_iteration_static(precision, _p(grid), n_dim, n_events, 5, 1, nat.VF_INT_SYMGAUSS,
                                       _p(good), 0, _p(out), _p(flags), nat.stream_handle())
    assert rc == nat.VF_OK, lib.vf_last_error_string()
    assert int(flags.item()) == 0
    res, sigma = out.cpu().numpy()
    assert abs(res - 1.0) < 6 * sigma
