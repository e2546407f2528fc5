"""Precision of the fp32 forms, stated against float64 on identical events.

* C2 (8-D Gaussian, 1e7 events, 3 trained iterations): the fused fp32 sampler
  on the same injected float64 uniforms the reference consumed in its own
  float64 run and in its float32 mode (``VEGASFLOW_FLOAT=32``, configflow.py:
  72-74), both recorded from the reference itself in
  ``tests/golden/c2_precision.npz``.  The fused form must stay within 0.05 sigma
  of the reference's float64 result each iteration.
* C3 (VegasFlowPlus adaptive, 6-D Breit-Wigner x linear, 2e6 events) and a
  subsample of C4 (the batched Gaussians): the fp32 samplers against the
  float64 oracle run on the kernels' own events -- the uniforms their Philox
  words stand for, u = (word + 1/2) / 2^32, on the same grid and event layout.
  Bar: |fp32 - fp64| < 0.05 sigma, a Monte Carlo sigma being what every result
  is reported with.
"""

import os

import numpy as np
import pytest
import torch

import oracle
from vegasflow_gb300 import VegasFlow, VegasFlowPlus, integrands
from vegasflow_gb300 import _native as nat
from vegasflow_gb300.batch import VegasBatch, c4_specs

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c2_precision.npz")
BAR = 0.05


def test_c2_fused_fp32_against_the_reference_float64_and_float32_modes():
    fx = np.load(GOLDEN)
    n, iters, floor = int(fx["n_events"]), int(fx["iterations"]), float(fx["raw_floor"])
    rng = np.random.default_rng(int(fx["seed"]))

    def source(m, d):  # the raw blocks the reference drew, in its chunk order
        return torch.as_tensor(oracle.tech_cut_affine(np.maximum(rng.random((m, d)), floor)), device="cuda")

    inst = VegasFlow(8, n, verbose=False, precision="fp32")
    inst.compile(integrands.symgauss(0.1))
    inst.set_uniform_source(source)
    got = np.array([[float(v) for v in inst._run_iteration()] for _ in range(iters)])
    h64, h32 = fx["f64/history"], fx["f32/history"]
    fused = (got[:, 0] - h64[:, 0]) / h64[:, 1]
    naive = (h32[:, 0] - h64[:, 0]) / h64[:, 1]
    print(f"C2 fused fp32 - fp64 (sigma units): {fused}; reference float32 mode: {naive}")
    assert np.all(np.abs(fused) < BAR), fused
    np.testing.assert_allclose(got[:, 1], h64[:, 1], rtol=0.02)


def test_c3_plus_fp32_against_oracle_on_its_own_events():
    n_dim, n_events, seed = 6, 2_000_000, 21
    coeffs = np.random.default_rng(3).random(5)
    inst = VegasFlowPlus(n_dim, n_events, adaptive=True, verbose=False, precision="fp32", seed=seed)
    inst.compile(integrands.breit_wigner(coeffs))
    orc = oracle.OraclePlus(n_dim, n_events, adaptive=True)
    assert (orc.n_strat, orc.n_hcubes) == (inst._n_strat, inst._n_hcubes)
    pulls = []
    for _ in range(3):
        # the oracle takes the GPU's grid and event layout: the same events
        orc.divisions = inst.divisions.cpu().numpy().copy()
        orc.n_ev = inst.n_ev.cpu().numpy().astype(np.int32)
        orc.n_events = int(orc.n_ev.sum())
        call = inst._call_ctr
        r32, s32 = (float(v) for v in inst._run_iteration())
        u = oracle.uniforms_of_words(oracle.philox_words(seed, call, 0, orc.n_events, n_dim))
        r64, s64 = orc.iteration(lambda m, d: u, lambda x: oracle.integrand_breit_wigner(x, coeffs=coeffs))
        pulls.append((r32 - r64) / s64)
        assert abs(s32 - s64) < 0.02 * s64
    print(f"C3 VEGAS+ fp32 - fp64 (sigma units): {pulls}")
    assert np.all(np.abs(pulls) < BAR), pulls


def _stream_words(seed, call, stream_id, n, n_dim):
    """The batched sampler's words: counter (ev, ev >> 32, call << 4 | q, stream id)."""
    ev = np.arange(n, dtype=np.uint64)
    key = (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    out = np.empty((n, 4 * ((n_dim + 3) // 4)), dtype=np.uint32)
    for q in range((n_dim + 3) // 4):
        r = oracle.philox4x32_10((ev & np.uint64(0xFFFFFFFF), ev >> np.uint64(32),
                                  np.uint64((call << 4) | q), np.uint64(stream_id)), key)
        for j in range(4):
            out[:, 4 * q + j] = r[j]
    return out[:, :n_dim]


def test_c4_batch_fp32_against_oracle_on_its_own_events():
    specs = c4_specs()
    # a subsample the oracle finishes quickly: resolvable integrals (>= 100
    # expected events in the peak on the uniform grid) of at most 2e6 events
    picks = []
    for i, (d, n, f) in enumerate(specs):
        p = np.asarray(f.params(d))
        mu, a = p[:d], p[d:]
        if n <= 2_000_000 and n * np.prod(a * np.sqrt(np.pi)) >= 100:
            picks.append(i)
    picks = picks[:12]
    assert len(picks) >= 6
    seed = 11
    b = VegasBatch([specs[i] for i in picks], seed=seed, stream_ids=picks)
    b.run(1)
    hist = b.history_host()[:, 0, :]
    pulls = []
    for k, i in enumerate(picks):
        d, n, f = specs[i]
        p = np.asarray(f.params(d))
        u = oracle.uniforms_of_words(_stream_words(seed, 0, i, n, d))
        orc = oracle.OracleVegas(d, n)
        pos = [0]

        def rows(m, dd):
            pos[0] += m
            return u[pos[0] - m: pos[0]]

        r64, s64 = orc.iteration(rows, lambda x: oracle.integrand_gauss_mu(x, p[:d], p[d:]))
        pulls.append((hist[k, 0] - r64) / s64)
    print(f"C4 batched fp32 - fp64 (sigma units) over {len(picks)} integrals: {np.round(pulls, 4)}")
    assert np.all(np.abs(pulls) < BAR), pulls


@pytest.mark.parametrize("which", ["prod", "symgauss"])
def test_high_dimension_fp32_against_float64_on_its_own_events(which):
    """16 dimensions, where an event's weight prod_d delta is ~50^-16: the fused
    fp32 sampler (its weight prescaled by a power of two) against the float64
    path on the same events (vf_philox_uniforms) and grid, every iteration of a
    trained run -- result and sigma."""
    n_dim, n, seed = 16, 2_000_000, 19
    f = integrands.prod() if which == "prod" else integrands.symgauss(0.3)
    f32 = VegasFlow(n_dim, n, verbose=False, precision="fp32", seed=seed)
    f32.compile(f)
    f64 = VegasFlow(n_dim, n, verbose=False, precision="fp64", seed=seed, events_limit=n)
    f64.compile(f)
    pulls = []
    for _ in range(4):
        grid, call = f32.divisions.clone(), f32._call_ctr
        r32, s32 = (float(v) for v in f32._run_iteration())
        u = torch.empty((n, n_dim), dtype=torch.float64, device="cuda")
        nat.call("vf_philox_uniforms", seed, call, call >> 28, 0, n, n_dim, nat.ptr(u), nat.stream_handle())
        f64.divisions.copy_(grid)
        f64.set_uniform_source(lambda m, d, u=u: u)
        r64, s64 = (float(v) for v in f64._run_iteration())
        assert s32 > 0 and abs(s32 - s64) < 0.02 * s64, (s32, s64)
        pulls.append((r32 - r64) / s64)
    print(f"16-D {which} fp32 - fp64 (sigma units): {pulls}")
    assert np.all(np.abs(pulls) < BAR), pulls
