"""The continuous-batching server: each request's result is the same alone and
in the mix (requests arriving while others run), and a short real-time run."""

import numpy as np
import pytest

from vegasflow_gb300 import integrands
from vegasflow_gb300.serving import Request, VegasServer, poisson_workload

pytestmark = pytest.mark.gpu


def _requests():
    rng = np.random.default_rng(4)
    c = rng.random(5)
    specs = [(4, 200_000, integrands.gauss([0.4, 0.5, 0.6, 0.45], [0.1, 0.12, 0.15, 0.2]), 0.0),
             (6, 300_000, integrands.breit_wigner(c), 0.0),
             (2, 20_000, integrands.symgauss(0.1), 0.0),
             (8, 1_000_000, integrands.symgauss(0.1), 0.0),
             (3, 50_000, integrands.prod(), 0.0),
             (5, 120_000, integrands.gauss(rng.uniform(0.3, 0.7, 5), rng.uniform(0.1, 0.2, 5)), 0.0)]
    return [Request(d, n, f, target_rel_sigma=2e-3, max_iterations=12, arrival=a, rid=i)
            for i, (d, n, f, a) in enumerate(specs)]


def test_same_result_alone_and_in_the_mix():
    """In the mix the requests join at different steps (admission in two waves)
    and leave when they converge; alone, each runs by itself.  Same Philox
    streams (seed, request id), same tiles: same iterations and results."""
    mix_reqs = _requests()
    server = VegasServer(max_slots=64, seed=99)
    for r in mix_reqs[:3]:
        server.submit(r)
    server._admit(0.0)
    server.step(lambda: 0.0)
    for r in mix_reqs[3:]:
        server.submit(r)
    while server.waiting or server.active:
        server._admit(0.0)
        server.step(lambda: 0.0)
    mix = {r.rid: r for r in server.done}
    assert len(mix) == len(mix_reqs)
    for r in _requests():
        alone = VegasServer(max_slots=4, seed=99)
        alone.run([r], realtime=False)
        got = alone.done[0]
        m = mix[r.rid]
        assert got.iterations == m.iterations
        np.testing.assert_allclose([got.result, got.sigma], [m.result, m.sigma], rtol=1e-5)


def test_results_against_exact():
    server = VegasServer(max_slots=64, seed=7)
    reqs = _requests()
    server.run(reqs, realtime=False)
    for r in server.done:
        if r.integrand.__name__ == "prod":
            ex = 0.5 ** r.n_dim
        elif r.integrand.__name__ == "symgauss":
            import math
            ex = math.erf(5.0) ** r.n_dim
        else:
            continue
        assert abs(r.result - ex) < 5 * r.sigma


def test_short_realtime_run():
    reqs = poisson_workload(rate=200.0, duration=2.0, seed=9)
    server = VegasServer(max_slots=2048, seed=1)
    m = server.run(reqs, realtime=True)
    assert m["requests"] == len(reqs) and m["flags"] == 0
    assert 0 < m["p50_latency_s"] <= m["p99_latency_s"] < 30.0
    assert m["events_per_s"] > 1e8
