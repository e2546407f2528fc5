"""The fp32 VEGAS map kernel (sampler API and the sampling half of
torch-evaluated iterations): bulk-copied tiles and plain stores write the same
bytes; its events are the fused sampler's events; x lies in the bin it reports."""

import numpy as np
import pytest
import torch

from vegasflow_gb300 import VegasFlow, integrands, _native as nat

pytestmark = pytest.mark.gpu


def _map(inst, n, call, offset_elems=0, with_ind=True):
    """x, w, ind from one map launch; `offset_elems` shifts the output arrays
    off 16-byte alignment (plain stores)."""
    d = inst.n_dim
    xb = torch.full((n * d + offset_elems,), -1.0, dtype=torch.float32, device="cuda")
    wb = torch.full((n + offset_elems,), -1.0, dtype=torch.float32, device="cuda")
    ib = torch.full((n * d + offset_elems,), -1, dtype=torch.int32, device="cuda")
    x, w, ind = xb[offset_elems:].view(n, d), wb[offset_elems:], ib[offset_elems:].view(n, d)
    inst._sample(n, 0, call, nat.VF_INT_NONE, None, False, False, ind=ind if with_ind else None, x=x, w=w)
    torch.cuda.synchronize()
    return x.clone(), w.clone(), ind.clone()


@pytest.mark.parametrize("n_dim", [1, 3, 8, 16])
@pytest.mark.parametrize("n", [1000, 70_000, 300_001])
def test_bulk_and_plain_stores_agree(n_dim, n):
    inst = VegasFlow(n_dim, n, verbose=False, precision="fp32", seed=9)
    inst.compile(integrands.symgauss(0.3))
    inst.run_integration(2)
    xa, wa, ia = _map(inst, n, 5)
    xp, wp, ip = _map(inst, n, 5, offset_elems=1)
    assert torch.equal(xa, xp) and torch.equal(wa, wp) and torch.equal(ia, ip)
    assert (wa > 0).all() and (ia >= 0).all() and (ia < 50).all()
    g = inst.divisions.cpu().numpy()
    x, ind = xa.cpu().numpy().astype(np.float64), ia.cpu().numpy()
    lo = np.take_along_axis(g, ind.T, axis=1).T
    hi = np.take_along_axis(g, ind.T + 1, axis=1).T
    assert np.all(x >= lo - 1e-6) and np.all(x <= hi + 1e-6)


def test_map_events_are_the_fused_samplers_events():
    """sum w f(x) over the map's events (torch, float64) equals the fused
    sampler's sum on the same Philox call to fp32 rounding."""
    n, call = 400_000, 11
    inst = VegasFlow(6, n, verbose=False, precision="fp32", seed=4)
    f = integrands.symgauss(0.2)
    inst.compile(f)
    inst.run_integration(3)
    x, w, _ = _map(inst, n, call, with_ind=False)
    res_torch = float((w.double() * f(x.double())).sum())
    inst._sample(n, 0, call, inst._int_id, inst._params_dev, False, False)
    inst._end_iteration(train=False, n_events=n, want_sums=True)
    res_fused = float(inst._workspace()["sums"][0])
    assert abs(res_torch - res_fused) <= 2e-5 * abs(res_fused)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("plus", [False, True])
def test_generate_random_array_normalisation_folded(precision, plus):
    """generate_random_array writes w already normalised (the Jacobian given to
    the sampler is xjac / (xjac n)); the same events through the raw sampler,
    divided as the reference divides (monte_carlo.py:245; vflowplus.py:182-183),
    agree to the precision's rounding."""
    from vegasflow_gb300 import VegasFlowPlus
    n_it, n = 200_000, 150_000
    inst = (VegasFlowPlus(3, n_it, verbose=False, precision=precision, seed=4) if plus
            else VegasFlow(3, n_it, verbose=False, precision=precision, seed=4))
    inst.compile(integrands.symgauss(0.3))
    inst.run_integration(2)
    ctr = inst._call_ctr
    x, p = inst.generate_random_array(n)
    inst._call_ctr = ctr
    xr, wr, *_ = inst._generate_random_array(n_it if plus else n)
    want = wr[:n] / (inst.xjac * n_it) * n_it / n if plus else wr / (inst.xjac * n)
    assert tuple(p.shape) == (n,) and p.dtype == want.dtype
    torch.testing.assert_close(x, xr[:n], rtol=0, atol=0)
    rtol = 4 * float(torch.finfo(p.dtype).eps)
    torch.testing.assert_close(p, want, rtol=rtol, atol=0)


def test_generate_random_array_weights():
    """generate_random_array's weights integrate the constant 1: sum over the
    events of xjac (= Jacobian / n) estimates the volume of the unit cube."""
    inst = VegasFlow(4, 1_000_000, verbose=False, precision="fp32", seed=2)
    inst.compile(integrands.symgauss(0.3))
    inst.run_integration(3)
    x, p = inst.generate_random_array(1_000_000)
    assert x.dtype == torch.float32 and tuple(x.shape) == (1_000_000, 4)
    vol = float(p.double().sum())
    assert abs(vol - 1.0) < 1e-2, vol
