"""CUDA-graph iterations (``cuda_graph=True``): one captured vf_iteration_dev
(VegasFlowPlus: vf_plus_iteration_dev) replayed per iteration, the Philox call
counter and the history row advancing on the device.  The replays run the same
kernels on the same events as the eager iterations, so results agree to the
histogram atomics' rounding."""

import ctypes
import math

import numpy as np
import pytest
import torch

from vegasflow_gb300 import PlainFlow, VegasFlow, VegasFlowPlus, integrands, _native as nat

pytestmark = pytest.mark.gpu

CAMEL = """
__device__ vf_real camel(const vf_real* x, int n_dim, vf_real weight, const double* p) {
  vf_real s1 = 0, s2 = 0;
  for (int d = 0; d < n_dim; ++d) {
    vf_real t1 = (x[d] - (vf_real)p[0]) / (vf_real)p[2], t2 = (x[d] - (vf_real)p[1]) / (vf_real)p[2];
    s1 += t1 * t1;
    s2 += t2 * t2;
  }
  return exp(-s1) + exp(-s2);
}
"""


def _pair(cls, precision, integrand, n_dim=4, n=100_000, **kw):
    out = []
    for graph in (False, True):
        inst = cls(n_dim, n, verbose=False, precision=precision, seed=17, cuda_graph=graph, **kw)
        inst.compile(integrand)
        out.append(inst)
    return out


# fp32: graph replays and eager launches run the same kernels on the same
# events, but the histogram's float atomics commit in whatever order the warps
# reach them, so the float32 refinement's grids (and the later iterations'
# results) agree to float32 rounding of the histogram, not bit for bit: the
# grid tolerance is the fp32 refinement's own (it agrees with the float64
# refinement to 2e-5).
FP32_GRID_ATOL = 2e-5


def _rtol(precision):
    return 1e-10 if precision == "fp64" else 1e-5


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_vegas_graph_matches_eager(precision):
    eager, graph = _pair(VegasFlow, precision, integrands.symgauss())
    for _ in range(2):  # the second run replays the same graph
        r_e = eager.run_integration(5)
        r_g = graph.run_integration(5)
        np.testing.assert_allclose(r_g, r_e, rtol=_rtol(precision))
    np.testing.assert_allclose(graph.divisions.cpu().numpy(), eager.divisions.cpu().numpy(), rtol=0,
                               atol=1e-12 if precision == "fp64" else FP32_GRID_ATOL)
    assert graph._call_ctr == eager._call_ctr == 10
    hist_e = [h[:2] for h in eager._history]
    hist_g = [h[:2] for h in graph._history]
    np.testing.assert_allclose(np.array(hist_g, dtype=float), np.array(hist_e, dtype=float), rtol=_rtol(precision))
    assert abs(r_g[0] - 1.0) < 5 * r_g[1]


def test_unrolled_graph_matches_eager():
    """11 iterations: one replay of an 8-iteration graph, then three replays of
    the one-iteration graph; the same history as eager launches."""
    from vegasflow_gb300.monte_carlo import GRAPH_UNROLL
    assert GRAPH_UNROLL == 8
    eager, graph = _pair(VegasFlow, "fp64", integrands.symgauss())
    r_e = eager.run_integration(11)
    r_g = graph.run_integration(11)
    np.testing.assert_allclose(r_g, r_e, rtol=1e-10)
    assert sorted(graph._graphs_unrolled) == [8]
    hist_e = np.array([h[:2] for h in eager._history], dtype=float)
    hist_g = np.array([h[:2] for h in graph._history], dtype=float)
    assert hist_g.shape == (11, 2)
    np.testing.assert_allclose(hist_g, hist_e, rtol=1e-10)
    np.testing.assert_allclose(graph.divisions.cpu().numpy(), eager.divisions.cpu().numpy(), rtol=0, atol=1e-12)


def test_graph_reused_and_recaptured_on_freeze():
    eager, graph = _pair(VegasFlow, "fp32", integrands.symgauss())
    eager.run_integration(3)
    graph.run_integration(3)
    g1 = graph._graph
    graph.run_integration(2)
    eager.run_integration(2)
    assert graph._graph is g1  # nothing changed: the same graph replays
    eager.freeze_grid()
    graph.freeze_grid()
    r_e = eager.run_integration(3)
    r_g = graph.run_integration(3)
    assert graph._graph is not g1  # training off: a new capture
    np.testing.assert_allclose(r_g, r_e, rtol=2e-6)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_plain_graph_matches_eager(precision):
    eager, graph = _pair(PlainFlow, precision, integrands.symgauss(0.3))
    np.testing.assert_allclose(graph.run_integration(4), eager.run_integration(4), rtol=_rtol(precision))


def test_jit_integrand_graph_matches_eager():
    f = integrands.cuda_integrand(CAMEL, "camel", params=[0.3, 0.7, 0.2])
    eager, graph = _pair(VegasFlow, "fp32", f, n_dim=3)
    np.testing.assert_allclose(graph.run_integration(4), eager.run_integration(4), rtol=2e-6)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("adaptive", [False, True])
def test_plus_graph_matches_eager(precision, adaptive):
    """VegasFlowPlus replays: the adaptive reallocation (n_ev, ev_start) stays on
    the device between iterations, and the host reads the new event count only
    when asked."""
    eager, graph = _pair(VegasFlowPlus, precision, integrands.symgauss(0.2), n_dim=3, n=200_000,
                         adaptive=adaptive)
    n0 = graph.n_events
    for _ in range(2):  # the second run replays the same graph
        r_e = eager.run_integration(4)
        r_g = graph.run_integration(4)
        np.testing.assert_allclose(r_g, r_e, rtol=_rtol(precision))
    g1 = graph._graph
    assert g1 is not None and graph._call_ctr == eager._call_ctr == 8 and len(graph._history) == 8
    np.testing.assert_allclose(graph.n_ev.cpu().numpy(), eager.n_ev.cpu().numpy(), rtol=0, atol=1)
    assert abs(graph.n_events - eager.n_events) <= graph.n_hypercubes
    if adaptive:
        assert graph.n_events != n0  # reallocated on the device
    np.testing.assert_allclose(graph.divisions.cpu().numpy(), eager.divisions.cpu().numpy(), rtol=0,
                               atol=1e-12 if precision == "fp64" else FP32_GRID_ATOL)
    graph.run_integration(2)
    assert graph._graph is g1  # reading n_events does not force a new capture
    assert abs(r_g[0] - math.erf(2.5) ** 3) < 5 * r_g[1]


def test_plus_jit_integrand_graph_matches_eager():
    f = integrands.cuda_integrand(CAMEL, "camel", params=[0.3, 0.7, 0.2])
    eager, graph = _pair(VegasFlowPlus, "fp32", f, n_dim=3, adaptive=True)
    np.testing.assert_allclose(graph.run_integration(4), eager.run_integration(4), rtol=2e-6)


def test_capture_survives_garbage_graphs():
    """Unreachable integrators that hold CUDA graphs (in reference cycles) do not
    break a later capture: the collector runs before it, never inside it (the
    reset of a graph is not permitted while a stream captures)."""
    import gc

    old = gc.get_threshold()
    try:
        for seed in range(3):
            a = VegasFlow(2, 10_000, verbose=False, seed=seed, cuda_graph=True)
            a.compile(integrands.symgauss())
            a.run_integration(2)
            a._cycle = a  # left to the cyclic collector
            del a
        gc.set_threshold(1, 1, 1)  # a collection at almost every allocation
        b = VegasFlow(2, 10_000, verbose=False, seed=7, cuda_graph=True)
        b.compile(integrands.symgauss())
        res, sig = b.run_integration(3)
        assert np.isfinite(res) and sig > 0
    finally:
        gc.set_threshold(*old)


def test_graph_grows_history():
    inst = VegasFlow(2, 20_000, verbose=False, seed=3, cuda_graph=True)
    inst.compile(integrands.symgauss())
    res, sig = inst.run_integration(40)  # more iterations than the initial history rows
    assert len(inst._history) == 40 and np.isfinite(res) and sig > 0


def test_history_full_flag():
    """vf_iteration_dev with no history row left records nothing and flags it."""
    inst = VegasFlow(2, 10_000, verbose=False, seed=3)
    inst.compile(integrands.symgauss())
    ws = inst._workspace()
    counters = torch.zeros(2, dtype=torch.int32, device="cuda")
    history = torch.zeros((1, 2), dtype=torch.float64, device="cuda")
    avg = torch.zeros(5, dtype=torch.float64, device="cuda")
    flags = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib = nat.load()
    for _ in range(2):
        nat.check(lib.vf_iteration_dev(nat.VF_ALG_VEGAS, nat.VF_PREC_F64, nat.ptr(inst.divisions), 2, 10_000,
                                       1e-4, None, None, 1.0, 3, nat.ptr(counters[0:1]), nat.ptr(counters[1:2]),
                                       nat.VF_INT_SYMGAUSS, nat.ptr(inst._params_dev), 1, 1.5,
                                       nat.ptr(ws["partials"]), inst._rows, nat.ptr(history), 1, nat.ptr(avg),
                                       nat.ptr(flags), nat.stream_handle()))
    torch.cuda.synchronize()
    assert counters.tolist() == [1, 1]  # the second call did not advance
    assert int(flags.item()) & nat.VF_FLAG_HISTORY_FULL
    assert history[0, 1].item() > 0


def test_nvtx_ranges_do_not_change_results(monkeypatch):
    """VEGASFLOW_NVTX=1 wraps iterations in NVTX ranges; results are unchanged."""
    out = []
    for flag in ("0", "1"):
        monkeypatch.setenv("VEGASFLOW_NVTX", flag)
        inst = VegasFlow(3, 50_000, verbose=False, precision="fp64", seed=8)
        inst.compile(integrands.symgauss())
        out.append(inst.run_integration(3))
    np.testing.assert_allclose(out[1], out[0], rtol=1e-12)
