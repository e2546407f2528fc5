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


USER_GAUSS_SRC = r"""
__device__ vf_real ugauss(const vf_real* x, int n_dim, vf_real weight, const double* p) {
  // prod_d exp(-((x_d - mu) / a)^2) / (a sqrt(pi)),  mu = p[0], a = p[1]
  const vf_real mu = (vf_real)p[0], a = (vf_real)p[1], norm = (vf_real)(0.5641895835477563 / p[1]);
  vf_real s = 0, f = 1;
  for (int d = 0; d < n_dim; ++d) {
    const vf_real t = (x[d] - mu) / a;
    s += t * t;
    f *= norm;
  }
  return f * exp(-s);
}
"""


def test_cuda_source_requests():
    """CUDA-source integrands as requests: compiled at submission, served by their
    own sampler launches (one per dimension class) beside built-in requests that
    arrive later; each result is within 5 sigma of the exact integral and the
    same alone as in the mix."""
    import math

    user = integrands.cuda_integrand(USER_GAUSS_SRC, "ugauss", params=[0.5, 0.2])

    def reqs():
        r = _requests()[:3]
        r += [Request(3, 100_000, user, target_rel_sigma=2e-3, max_iterations=10, rid=10),
              Request(11, 300_000, user, target_rel_sigma=2e-3, max_iterations=10, rid=11)]
        return r

    mix_reqs = reqs()
    server = VegasServer(max_slots=64, seed=41)
    for r in mix_reqs[3:]:
        assert server.submit(r)
    assert mix_reqs[3].program != mix_reqs[4].program  # a sampler build per dimension class
    server._admit(0.0)
    server.step(lambda: 0.0)
    for r in mix_reqs[:3]:
        server.submit(r)
    while server.waiting or server.active:
        server._admit(0.0)
        server.step(lambda: 0.0)
    mix = {r.rid: r for r in server.done}
    assert len(mix) == 5 and all(r.status in ("converged", "finished") for r in mix.values())
    for rid in (10, 11):
        r = mix[rid]
        assert abs(r.result - math.erf(2.5) ** r.n_dim) < 5 * r.sigma, (rid, r.result, r.sigma)
    for r in reqs()[3:]:
        alone = VegasServer(max_slots=4, seed=41)
        alone.run([r], realtime=False)
        got = alone.done[0]
        m = mix[r.rid]
        assert got.iterations == m.iterations
        np.testing.assert_allclose([got.result, got.sigma], [m.result, m.sigma], rtol=1e-5)


def test_short_realtime_run():
    reqs = poisson_workload(rate=200.0, duration=2.0, seed=9)
    server = VegasServer(max_slots=2048, seed=1)
    m = server.run(reqs, realtime=True)
    assert m["requests"] == len(reqs) and m["flags"] == 0
    assert 0 < m["p50_latency_s"] <= m["p99_latency_s"] < 30.0
    assert m["events_per_s"] > 1e8


def _drive(server, steps, now=0.0):
    """Advance the server by hand: triage, admission, one step each."""
    for _ in range(steps):
        server._triage(now)
        server._admit(now)
        if server.active:
            server.step(lambda: now)


def test_status_rows_are_the_slot_state():
    """The iteration end writes each active request's (mean, sigma, iterations)
    into the server's pinned status array, in the order of the step's items:
    after every step they equal the slots' device state, and requests joining
    and leaving reorder the items."""
    server = VegasServer(max_slots=32, hbm_budget=1e9, seed=5)
    reqs = [Request(d, n, integrands.symgauss(0.2), target_rel_sigma=1e-12, max_iterations=50, rid=i)
            for i, (d, n) in enumerate([(3, 20_000), (9, 200_000), (5, 1_000_000), (12, 50_000)])]
    for r in reqs[:3]:
        server.submit(r)
    for k in range(4):
        if k == 2:
            server.submit(reqs[3])
            server.cancel(reqs[1].rid)
        _drive(server, 1)
        avg = server.avg.cpu().numpy()
        iters = server.iters.cpu().numpy()
        for r in server.active:
            assert r.result == avg[r.slot, 2] and r.sigma == avg[r.slot, 3]
            assert r.iterations == iters[r.slot]
    assert reqs[1].status == "cancelled" and reqs[3].iterations == 2


def test_reused_request_id_gets_its_own_tables():
    """A request id used again (the caller's choice) with another size: the
    step's cached tables are rebuilt, so the second request's result equals the
    same request served by a fresh server (one iteration: bit for bit, since
    only the refinement after it depends on the order of the histogram's float
    atomics)."""
    def serve(server, req, steps):
        server.submit(req)
        _drive(server, steps)
        return req

    a = Request(3, 30_000, integrands.symgauss(0.2), target_rel_sigma=1e-12, max_iterations=1, rid=7)
    b = Request(5, 60_000, integrands.symgauss(0.2), target_rel_sigma=1e-12, max_iterations=1, rid=7)
    shared = VegasServer(max_slots=8, hbm_budget=1e9, seed=4)
    serve(shared, a, 3)
    assert a.status == "finished"
    serve(shared, b, 3)
    b_alone = serve(VegasServer(max_slots=8, hbm_budget=1e9, seed=4),
                    Request(5, 60_000, integrands.symgauss(0.2), target_rel_sigma=1e-12, max_iterations=1, rid=7), 3)
    assert b.status == b_alone.status == "finished"
    assert b.result == b_alone.result and b.sigma == b_alone.sigma


def test_rejections_do_not_stop_the_server():
    server = VegasServer(max_slots=64, hbm_budget=2e7, seed=3)
    good = Request(3, 50_000, integrands.symgauss(0.2), target_rel_sigma=1e-9, max_iterations=3, rid=0)
    bad = [Request(17, 1000, integrands.symgauss(), rid=1),                                   # dimensions
           Request(2, 1, integrands.symgauss(), rid=2),                                       # events
           Request(4, 1000, integrands.cuda_integrand("__device__ vf_real f(const vf_real* x, int n, "
                                                     "vf_real w, const double* p) { return y[0]; }",
                                                     "f"), rid=3),                            # does not compile
           Request(3, 1000, integrands.gauss([0.5, 0.5], [0.1, 0.1]), rid=4),                 # params for 2-D
           Request(16, 10 ** 9, integrands.symgauss(), rid=5)]                               # over the budget
    assert server.submit(good)
    for r in bad:
        assert not server.submit(r)
        assert r.status == "rejected" and r.error
    assert "did not compile" in bad[2].error
    _drive(server, 4)
    assert good.status == "finished" and good.iterations == 3


def test_cancel_waiting_and_active():
    server = VegasServer(max_slots=2, hbm_budget=1e9, seed=5)
    reqs = [Request(4, 100_000, integrands.symgauss(0.2), target_rel_sigma=1e-9, max_iterations=10, rid=i)
            for i in range(3)]
    for r in reqs:
        server.submit(r)
    _drive(server, 2)  # two slots: requests 0 and 1 active, 2 waiting
    assert [r.status for r in reqs] == ["active", "active", "waiting"]
    server.cancel(1)
    server.cancel(2)
    _drive(server, 1)
    assert reqs[1].status == "cancelled" and reqs[2].status == "cancelled"
    assert reqs[1].iterations == 2 and np.isfinite(reqs[1].result)  # its result so far is kept
    _drive(server, 10)
    assert reqs[0].status == "finished" and reqs[0].iterations == 10


def test_expiry():
    server = VegasServer(max_slots=8, hbm_budget=1e9, seed=6)
    slow = Request(4, 100_000, integrands.symgauss(0.2), target_rel_sigma=1e-9, max_iterations=50, rid=0,
                   arrival=0.0, timeout=1.0)
    server.submit(slow)
    _drive(server, 3, now=0.5)
    assert slow.status == "active" and slow.iterations == 3
    _drive(server, 1, now=1.5)
    assert slow.status == "expired" and slow.iterations == 3 and "timed out" in slow.error
    assert server.free_slots and server.bytes_in_use == 0


def test_allocation_failures_fail_only_their_requests():
    """Host-side fault injection: an admission whose slot set-up fails, and a
    partial-row buffer that cannot grow, fail the requests concerned; the
    others are served."""
    state = {"admit": 1, "grow": 1}

    def hook(event, **info):
        if state.get(event, 0) > 0:
            state[event] -= 1
            raise MemoryError(f"injected {event} failure")

    server = VegasServer(max_slots=16, hbm_budget=1e9, seed=7, fault_hook=hook)
    # one request's rows (20,000 events in 10 tiles of 2,048: 10 x 152 doubles) fit, two do not
    server.partials = server.partials[:2000]
    first = [Request(3, 20_000, integrands.symgauss(0.2), max_iterations=2, rid=i) for i in range(2)]
    for r in first:
        server.submit(r)
    _drive(server, 1)  # the admission fails
    assert all(r.status == "failed" and "admission failed" in r.error for r in first)
    assert server.bytes_in_use == 0 and len(server.free_slots) == 16
    second = [Request(3, 20_000, integrands.symgauss(0.2), max_iterations=2, rid=10 + i) for i in range(3)]
    for r in second:
        server.submit(r)
    _drive(server, 3)  # the buffer cannot grow: the newest requests fail until the rest fit
    failed = [r for r in second if r.status == "failed"]
    served = [r for r in second if r.status in ("converged", "finished")]
    assert failed and all("allocation failed" in r.error for r in failed)
    assert len(failed) + len(served) == 3
