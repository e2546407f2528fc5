"""Injected float64 uniforms in the fused fp32 sampler: the TMA-staged path
(tiles of one event per thread copied into swizzled shared memory, D = 4, 8, 16,
16-byte aligned arrays) and the plain-load path (any D, any alignment) see the
same events, so they give the same sums and histogram to float rounding, and
both agree with the float64 oracle's bins on the initial grid."""

import numpy as np
import pytest
import torch

import oracle
from vegasflow_gb300 import VegasFlow, integrands

pytestmark = pytest.mark.gpu


def _uniforms(n, n_dim, seed, misalign):
    u = oracle.tech_cut_affine(np.random.default_rng(seed).random((n, n_dim)))
    if not misalign:
        return torch.as_tensor(u, device="cuda").contiguous()
    # an array starting 8 bytes past a 16-byte boundary takes the plain-load path
    buf = torch.empty(n * n_dim + 1, dtype=torch.float64, device="cuda")
    view = buf[1:].view(n, n_dim)
    view.copy_(torch.as_tensor(u, device="cuda"))
    assert view.data_ptr() % 16 == 8
    return view


def _one_pass(inst, u, train=True):
    """One sampler launch on `u` and the iteration end; (res, res2) and arr_res2."""
    n = u.shape[0]
    inst._sample(n, 0, 0, inst._int_id, inst._params_dev, train, False, u_inj=u)
    inst._end_iteration(train=False, n_events=n, want_hist=True, want_sums=True)
    ws = inst._workspace()
    flags = int(ws["flags"][0].item())
    return ws["sums"].cpu().numpy().copy(), ws["hist"].cpu().numpy().copy(), flags


@pytest.mark.parametrize("n_dim", [4, 8, 16, 6])
@pytest.mark.parametrize("n", [1000, 300_001, 3_000_000])
def test_tma_and_plain_paths_agree(n_dim, n):
    inst = VegasFlow(n_dim, n, verbose=False, precision="fp32", seed=1)
    inst.compile(integrands.symgauss(0.3))
    inst.run_integration(2)  # a trained, non-uniform grid
    aligned = _uniforms(n, n_dim, 5, misalign=False)
    shifted = _uniforms(n, n_dim, 5, misalign=True)
    s_a, h_a, f_a = _one_pass(inst, aligned)
    s_p, h_p, f_p = _one_pass(inst, shifted)
    assert f_a == 0 and f_p == 0
    np.testing.assert_allclose(s_a, s_p, rtol=2e-6)
    scale = h_p.sum(axis=1, keepdims=True)
    np.testing.assert_allclose(h_a / scale, h_p / scale, rtol=0, atol=1e-6)


def test_tma_path_bins_match_oracle():
    """On the initial grid the fp32 integral of the injected events matches the
    float64 oracle's iteration on the same uniforms to a small fraction of sigma
    (the bins are exact; x is rounded to fp32)."""
    n_dim, n = 8, 2_000_000
    u = oracle.tech_cut_affine(np.random.default_rng(11).random((n, n_dim)))
    orc = oracle.OracleVegas(n_dim, n)
    pos = [0]

    def rows(m, d):  # consecutive chunks, as the oracle asks for them
        pos[0] += m
        return u[pos[0] - m: pos[0]]

    ref = orc.iteration(rows, lambda x: oracle.integrand_symgauss(x, 0.1))
    assert pos[0] == n
    inst = VegasFlow(n_dim, n, verbose=False, precision="fp32", events_limit=n)
    inst.compile(integrands.symgauss())
    ud = torch.as_tensor(u, device="cuda").contiguous()
    assert ud.data_ptr() % 16 == 0
    inst.set_uniform_source(lambda m, d: ud)
    r, s = (float(v) for v in inst._run_iteration())
    assert abs(r - ref[0]) < 0.01 * ref[1], (r, ref)
    assert abs(s - ref[1]) < 0.01 * ref[1], (s, ref)


def test_uniforms_outside_unit_interval_flagged_on_tma_path():
    """Out-of-range injected values take the float64 operations inside the TMA
    path too: clamped into the grid and flagged, never read out of bounds."""
    n_dim, n = 8, 4096
    u = torch.full((n, n_dim), 0.5, dtype=torch.float64, device="cuda")
    u[7, 3] = 1.5
    u[100, 0] = -0.25
    inst = VegasFlow(n_dim, n, verbose=False, precision="fp32")
    inst.compile(integrands.symgauss())
    _, _, flags = _one_pass(inst, u)
    assert flags & 1
