"""VegasFlowPlus on the GPU: the reference's runs replayed, the Philox stream
against the oracle, the C3 configuration, and the reference's VEGAS+ tests."""

import numpy as np
import pytest
import torch

import oracle
from conftest import raw_blocks
from vegasflow_gb300 import VegasFlowPlus, integrands

pytestmark = pytest.mark.gpu


def _replay(golden, name):
    blocks = [torch.as_tensor(oracle.tech_cut_affine(b), device="cuda") for b in raw_blocks(golden, name)]
    it = iter(blocks)
    return lambda n, d: next(it)


@pytest.mark.parametrize("case,kind", [("plus2", "device"), ("plus2", "torch"),
                                       ("plus3_adaptive", "device"), ("plus3_adaptive", "torch")])
def test_reference_plus_runs_replayed(golden, case, kind):
    n_dim, n_events, adaptive, n_iter = {"plus2": (2, 2000, False, 2),
                                         "plus3_adaptive": (3, 4000, True, 3)}[case]
    inst = VegasFlowPlus(n_dim, n_events, adaptive=adaptive, verbose=False)
    f = integrands.symgauss()
    inst.compile(f if kind == "device" else f.__call__)
    inst.set_uniform_source(_replay(golden, case))
    hist, grids, n_evs = [], [], []
    for _ in range(n_iter):
        n_evs.append(inst.n_ev.cpu().numpy().copy())
        r, s = inst._run_iteration()
        hist.append((float(r), float(s)))
        grids.append(inst.divisions.cpu().numpy().copy())
    np.testing.assert_allclose(np.array(hist), golden[f"{case}/history"], rtol=1e-10)
    np.testing.assert_allclose(np.stack(grids), golden[f"{case}/grids"], rtol=0, atol=1e-13)
    np.testing.assert_array_equal(np.stack(n_evs), golden[f"{case}/n_ev"])


def test_plus_philox_against_oracle():
    """Adaptive VEGAS+ with the in-kernel stream: every iteration, the reallocated
    n_ev and the grids against the oracle fed the same Philox uniforms."""
    n_dim, n_events, seed, n_iter = 4, 200_000, 21, 4
    c = np.random.default_rng(3).random(n_dim - 1)
    inst = VegasFlowPlus(n_dim, n_events, adaptive=True, verbose=False, seed=seed)
    inst.compile(integrands.breit_wigner(c))
    orc = oracle.OraclePlus(n_dim, n_events, adaptive=True)
    calls = iter(range(n_iter))
    src = lambda m, d: oracle.uniforms_f64_philox(seed, next(calls), 0, m, d)  # noqa: E731
    for _ in range(n_iter):
        r, s = (float(v) for v in inst._run_iteration())
        ref = orc.iteration(src, lambda x: oracle.integrand_breit_wigner(x, coeffs=c))
        np.testing.assert_allclose([r, s], ref, rtol=1e-9)
        np.testing.assert_array_equal(inst.n_ev.cpu().numpy(), orc.n_ev)
        assert inst.n_events == orc.n_events
        np.testing.assert_allclose(inst.divisions.cpu().numpy(), orc.divisions, rtol=0, atol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_c3_breit_wigner_adaptive(precision):
    """C3: 6-D Breit-Wigner x linear, 2e6 events, adaptive, 10 iterations."""
    c = np.random.default_rng(3).random(5)
    inst = VegasFlowPlus(6, 2_000_000, adaptive=True, verbose=False, precision=precision, seed=5)
    inst.compile(integrands.breit_wigner(c))
    res, sigma = inst.run_integration(10)
    exact = oracle.breit_wigner_exact(6, coeffs=c)
    assert sigma < 1e-3 * exact
    assert abs(res - exact) < 4 * sigma, (res, sigma, exact)


dim, ncalls, n_iter = 2, np.int32(1e4), 4


def example_integrand(xarr, weight=None):
    n_dim = xarr.shape[-1]
    a = 0.1
    n100 = float(100 * n_dim)
    pref = (1.0 / a / np.sqrt(np.pi)) ** n_dim
    coef = torch.sum(torch.arange(n100 + 1, dtype=xarr.dtype, device=xarr.device))
    coef = coef + torch.sum(((xarr - 0.5) / a) ** 2, dim=1)
    coef = coef - (n100 + 1) * n100 / 2.0
    return pref * torch.exp(-coef)


def check_is_one(result, sigmas=3, target=1.0):
    np.testing.assert_allclose(result[0], target, atol=np.mean(result[1] * sigmas))


@pytest.mark.parametrize("mode", range(4))
def test_VegasFlowPlus_ADAPTIVE_SAMPLING(mode):
    """test_algs.py:209-214."""
    fns = {0: example_integrand,
           1: lambda xarr, n_dim=None: example_integrand(xarr),
           2: lambda xarr: example_integrand(xarr),
           3: lambda xarr, n_dim=None, weight=None: example_integrand(xarr)}
    inst = VegasFlowPlus(dim, ncalls, verbose=False, seed=20, adaptive=True)
    inst.compile(fns[mode])
    check_is_one(inst.run_integration(n_iter))


def test_VegasFlowPlus_NOT_ADAPTIVE_SAMPLING():
    """test_algs.py:217-222."""
    inst = VegasFlowPlus(dim, ncalls, adaptive=False, verbose=False, seed=21)
    inst.compile(example_integrand)
    check_is_one(inst.run_integration(n_iter))


def test_rng_generation_vegasflowplus(n_events=100):
    inst = VegasFlowPlus(dim, ncalls, verbose=False, seed=22)
    inst.compile(example_integrand)
    rnds, px = inst.generate_random_array(n_events)
    assert tuple(rnds.shape) == (n_events, dim) and tuple(px.shape) == (n_events,)


def test_notworking_vectorial():
    with pytest.raises(NotImplementedError):
        inst = VegasFlowPlus(dim, ncalls, verbose=False, seed=23)
        inst.compile(lambda x: torch.exp(-((x - 1.0) ** 4)))


def test_plus_integration_limits():
    rng = np.random.default_rng(23)
    dims = 3
    xmin = -1.0 + rng.random(dims) * 2.0
    xmax = 3.0 + rng.random(dims)
    inst = VegasFlowPlus(dims, 20_000, xmin=xmin, xmax=xmax, verbose=False, seed=24)
    inst.compile(integrands.prod())
    res = inst.run_integration(5)
    expected = np.prod(np.array(xmax) ** 2 / 2 - np.array(xmin) ** 2 / 2)
    check_is_one(res, target=expected)
