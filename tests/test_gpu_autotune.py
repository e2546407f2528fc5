"""Launch-shape autotuner on the GPU: every launch shape gives the same
integral (the Philox stream is per event, so only summation order and the
histogram's float atomics differ), and ``autotune=True`` picks one, caches it
and integrates correctly with it."""

import numpy as np
import pytest
import torch

from vegasflow_gb300 import VegasFlow, autotune, integrands

pytestmark = pytest.mark.gpu

N_DIM = 6
N_EVENTS = 2_000_000


def _run(shape, n_iter=3, train=True, seed=123):
    inst = VegasFlow(N_DIM, N_EVENTS, precision="fp32", seed=seed, verbose=False, train=train)
    inst.compile(integrands.symgauss())
    inst.set_launch_shape(shape)
    first = inst.run_integration(1)
    res, sig = inst.run_integration(n_iter)
    return first, res, sig, inst


@pytest.mark.parametrize("shape", [autotune.LaunchShape(512, 0, 0), autotune.LaunchShape(512, 1, 0),
                                   autotune.LaunchShape(1024, 0, 0)])
def test_shapes_agree(shape):
    (r0, s0), res0, sig0, _ = _run(None)
    (r1, s1), res1, sig1, inst = _run(shape)
    assert inst.launch_shape == shape
    # first iteration: identical events on the initial grid, different summation order
    assert abs(r1 - r0) <= 1e-6 * abs(r0)
    assert abs(s1 - s0) <= 1e-4 * s0
    # later iterations: the grid refines from histograms that differ by float rounding
    assert abs(res1 - res0) < 0.5 * sig0
    assert abs(res1 - 1.0) < 5 * sig1


def test_frozen_grid_shapes_agree():
    (r0, _), res0, _, _ = _run(None, train=False)
    (r1, _), res1, _, _ = _run(autotune.LaunchShape(512, 1, 0), train=False)
    assert abs(r1 - r0) <= 1e-6 * abs(r0)
    assert abs(res1 - res0) <= 1e-6 * abs(res0)


def test_autotune_picks_and_caches(tmp_path, monkeypatch):
    path = tmp_path / "shapes.json"
    monkeypatch.setenv("VEGASFLOW_GB300_TUNE_CACHE", str(path))
    saved = autotune.current()
    inst = VegasFlow(N_DIM, N_EVENTS, precision="fp32", seed=5, verbose=False, autotune=True)
    inst.compile(integrands.symgauss())
    shape = inst.launch_shape
    assert shape in autotune.candidates(train=True)
    assert autotune.current() == shape  # applied for this integrator's launches
    cache = autotune.TuneCache(str(path))
    assert len(cache.entries) == 1
    entry = next(iter(cache.entries.values()))
    assert entry["ms"] <= entry["default_ms"] * 1.0001
    res, sig = inst.run_integration(4)
    assert abs(res - 1.0) < 5 * sig
    # a second integrator of the same workload reads the cache (no re-timing)
    cache_mtime = path.stat().st_mtime_ns
    again = VegasFlow(N_DIM, N_EVENTS, precision="fp32", seed=6, verbose=False, autotune=True)
    again.compile(integrands.symgauss())
    assert again.launch_shape == shape
    assert path.stat().st_mtime_ns == cache_mtime
    # an untuned integrator interleaved with it runs on the default shape
    plain = VegasFlow(N_DIM, N_EVENTS, precision="fp32", seed=7, verbose=False)
    plain.compile(integrands.symgauss())
    plain.run_integration(1)
    assert autotune.current() == autotune.DEFAULT_SHAPE
    again.run_integration(1)
    assert autotune.current() == shape
    autotune.apply(saved)


def test_autotune_is_noop_off_the_fused_path(tmp_path, monkeypatch):
    monkeypatch.setenv("VEGASFLOW_GB300_TUNE_CACHE", str(tmp_path / "s.json"))
    inst = VegasFlow(2, 10_000, precision="fp64", seed=1, verbose=False, autotune=True)
    inst.compile(integrands.symgauss())
    assert inst.launch_shape is None
    assert not (tmp_path / "s.json").exists()


def _hist(inst, generic=False):
    """One sampling pass on the current grid (always the same Philox call, so
    the same events); the (n_dim, 50) arr_res2 it fills.  ``generic``: through
    the generic fp32 sampler (a point tap routes the launch there), whose
    histogram is a plain per-dimension table in bin order."""
    n = inst.n_events
    inst._workspace()["flags"].zero_()
    if generic:
        x = torch.empty((n, inst.n_dim), dtype=torch.float32, device="cuda")
        inst._sample(n, 0, 1000, inst._int_id, inst._params_dev, True, False, x=x)
    else:
        inst._apply_shape()
        inst._sample(n, 0, 1000, inst._int_id, inst._params_dev, True, False)
    inst._end_iteration(train=False, want_hist=True)
    assert int(inst._workspace()["flags"][0].item()) == 0
    return inst._workspace()["hist"].cpu().numpy().copy()


@pytest.mark.parametrize("n_dim", [1, 3, 8, 12])
@pytest.mark.parametrize("trained", [False, True])
def test_histogram_matches_generic_sampler(n_dim, trained):
    """The fused sampler's joint pair tables (reversed, swizzled cells) give
    every dimension the per-bin sums of the generic sampler's plain table on the
    same events and grid, under both block sizes (float rounding apart).  (The
    generic sampler keeps the weight without its 50^D factor in float32, whose
    square underflows beyond about 12 dimensions; 16 dimensions are checked
    against the float64 path in test_gpu_precision.py.)"""
    inst = VegasFlow(n_dim, 1_000_000, precision="fp32", seed=4, verbose=False)
    # a width at which no event's (w f)^2 underflows float32 on the uniform grid
    # in either sampler (the generic one evaluates the normalised integrand)
    inst.compile(integrands.symgauss(0.3))
    if trained:
        inst.run_integration(4)
    ref = _hist(inst, generic=True)
    assert np.all(np.isfinite(ref)) and ref.sum() > 0
    scale = ref.sum(axis=1, keepdims=True)
    for shape in (autotune.LaunchShape(1024, 0, 0), autotune.LaunchShape(512, 0, 0)):
        inst.set_launch_shape(shape)
        h = _hist(inst)
        np.testing.assert_allclose(h / scale, ref / scale, rtol=0, atol=2e-5, err_msg=str(shape))
