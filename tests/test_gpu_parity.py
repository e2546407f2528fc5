"""GPU parity: the CUDA path against the oracle and the reference's golden runs.

Bars: bin indices, points and weights bit-exact in float64 (injected uniforms
and the Philox stream); integrals, sigmas and refined grids to 1e-10 relative
(only the summation order differs); fp32 fused form within its Monte Carlo
sigma of the float64 oracle on the same injected uniforms."""

import numpy as np
import pytest
import torch

import oracle
from conftest import raw_blocks
from vegasflow_gb300 import PlainFlow, VegasFlow, integrands
from vegasflow_gb300 import _native as nat
from vegasflow_gb300.utils import consume_array_into_indices

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def symgauss_np(x):
    return oracle.integrand_symgauss(x, 0.1)


class chunked:
    """Uniform source handing out consecutive rows of ``arr``, one events_limit
    chunk per call (the order in which the iteration consumes them)."""

    def __init__(self, arr):
        self.arr = arr
        self.pos = 0

    def __call__(self, m, d):
        blk = self.arr[self.pos:self.pos + m]
        self.pos += m
        return blk


def test_map_bit_exact_against_reference(golden):
    """vflow.py:93-126 on the reference's own uniforms and trained grid."""
    grid = golden["map/grid"]
    inst = VegasFlow(grid.shape[0], 10, verbose=False)
    inst.load_grid(numpy_grid=grid)
    x, w, ind = inst._digest_random_generation(dev(golden["map/rnds"]))
    np.testing.assert_array_equal(ind.cpu().numpy(), golden["map/ind"])
    np.testing.assert_array_equal(x.cpu().numpy(), golden["map/x"])
    np.testing.assert_array_equal(w.cpu().numpy(), golden["map/w"])


def test_philox_stream_bit_exact_against_oracle():
    """The in-kernel Philox4x32-10 stream + map, event by event."""
    n_dim, n, seed = 5, 20_000, 1234
    inst = VegasFlow(n_dim, 100_000, verbose=False, seed=seed)
    rng = np.random.default_rng(3)
    grid = np.sort(rng.random((n_dim, 51)), axis=1)
    grid[:, 0], grid[:, -1] = 0.0, 1.0
    inst.load_grid(numpy_grid=grid)
    inst.compile(integrands.symgauss())
    inst._call_ctr = 5
    x, w, ind = inst._generate_random_array(n)
    u = oracle.uniforms_f64_philox(seed, 5, 0, n, n_dim)
    ox, ow, oind = oracle.vegas_map(u, grid)
    np.testing.assert_array_equal(ind.cpu().numpy(), oind)
    np.testing.assert_array_equal(x.cpu().numpy(), ox)
    np.testing.assert_array_equal(w.cpu().numpy(), ow * (1.0 / 100_000))


def test_refine_against_reference(golden):
    for t_res, sub, want in zip(golden["refine/in"], golden["refine/sub"], golden["refine/out"]):
        inst = VegasFlow(1, 10, verbose=False)
        inst.load_grid(numpy_grid=sub[None, :])
        inst.refine_grid(dev(t_res[None, :]))
        np.testing.assert_allclose(inst.divisions.cpu().numpy()[0], want, rtol=1e-12, atol=1e-15)


def test_consume_array_into_indices(golden):
    got = consume_array_into_indices(dev(golden["consume/in"]), dev(golden["consume/idx"], torch.int32), 50)
    np.testing.assert_allclose(got.cpu().numpy(), golden["consume/out"], rtol=1e-12)
    # empty input and a single bin
    empty = consume_array_into_indices(dev(np.zeros(0)), dev(np.zeros(0), torch.int32), 7)
    np.testing.assert_array_equal(empty.cpu().numpy(), np.zeros(7))


def _replay(golden, name):
    blocks = [dev(oracle.tech_cut_affine(b)) for b in raw_blocks(golden, name)]
    it = iter(blocks)
    return lambda n, d: next(it)


def _quirky(xarr, weight=None):
    n_dim = xarr.shape[-1]
    n100 = 100.0 * n_dim
    coef = torch.sum(torch.arange(n100 + 1, dtype=torch.float64))
    coef = coef + torch.sum(((xarr - 0.5) / 0.1) ** 2, dim=1)
    coef = coef - (n100 + 1) * n100 / 2.0
    return (1.0 / 0.1 / np.sqrt(np.pi)) ** n_dim * torch.exp(-coef)


REPLAYS = {
    "vegas4": (lambda g: VegasFlow(4, 2000, verbose=False), integrands.symgauss(), 3, None),
    "vegas4_chunks": (lambda g: VegasFlow(4, 1500, events_limit=400, verbose=False),
                      integrands.symgauss(), 2, None),
    "vegas4_torch": (lambda g: VegasFlow(4, 2000, verbose=False), integrands.symgauss().__call__, 3, None),
    "vegas2_quirky": (lambda g: VegasFlow(2, 1000, verbose=False), _quirky, 3, None),
    "vegas_limits": (lambda g: VegasFlow(3, 1200, xmin=g["vegas_limits/xmin"], xmax=g["vegas_limits/xmax"],
                                         verbose=False), integrands.prod(), 2, None),
    "vegas_freeze": (lambda g: VegasFlow(3, 1000, verbose=False), integrands.symgauss(), 3, 2),
    "plain3": (lambda g: PlainFlow(3, 1500, verbose=False), integrands.symgauss(), 2, None),
    "plain3_torch": (lambda g: PlainFlow(3, 1500, verbose=False), integrands.symgauss().__call__, 2, None),
}


@pytest.mark.parametrize("case", sorted(REPLAYS))
def test_reference_runs_replayed_through_api(golden, case):
    """The reference's runs (tests/golden) replayed through the public API on the
    same uniforms: per-iteration (res, sigma), final, grids; first-chunk taps."""
    make, integrand, n_iter, freeze_after = REPLAYS[case]
    name = case.replace("_torch", "")
    inst = make(golden)
    inst.compile(integrand)
    inst.set_uniform_source(_replay(golden, name))
    hist, grids = [], []
    for it in range(n_iter):
        if freeze_after is not None and it == freeze_after:
            inst.freeze_grid()
        r, s = inst._run_iteration()
        hist.append((float(r), float(s)))
        if hasattr(inst, "divisions"):
            grids.append(inst.divisions.cpu().numpy().copy())
    np.testing.assert_allclose(np.array(hist), golden[f"{name}/history"], rtol=RTOL)
    np.testing.assert_allclose(oracle.weighted_average(hist), golden[f"{name}/final"], rtol=RTOL)
    if grids:
        np.testing.assert_allclose(np.stack(grids), golden[f"{name}/grids"], rtol=0, atol=1e-13)


def test_run_integration_average_matches_reference(golden):
    inst = VegasFlow(4, 2000, verbose=False)
    inst.compile(integrands.symgauss())
    inst.set_uniform_source(_replay(golden, "vegas4"))
    res, sigma = inst.run_integration(3)
    np.testing.assert_allclose([res, sigma], golden["vegas4/final"], rtol=RTOL)
    assert len(inst.history) == 3
    np.testing.assert_allclose(np.array([h[:2] for h in inst.history], dtype=float),
                               golden["vegas4/history"], rtol=RTOL)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("alg", ["vegas", "plain"])
def test_fused_matches_torch_path(alg, precision):
    """Same Philox stream through the fused device integrand and the unfused torch
    callable: float64 equal to rounding, fp32 to fp32 rounding."""
    cls = VegasFlow if alg == "vegas" else PlainFlow
    out = []
    for f in (integrands.symgauss(), integrands.symgauss().__call__):
        inst = cls(3, 50_000, verbose=False, seed=99, precision=precision, events_limit=20_000)
        inst.compile(f)
        out.append(np.array([[float(v) for v in inst._run_iteration()] for _ in range(3)]))
    tol = 1e-11 if precision == "fp64" else 2e-5
    np.testing.assert_allclose(out[0], out[1], rtol=tol)


def test_fp64_philox_iterations_against_oracle():
    n_dim, n, seed = 4, 200_000, 7
    inst = VegasFlow(n_dim, n, verbose=False, seed=seed)
    inst.compile(integrands.symgauss())
    got = [tuple(float(v) for v in inst._run_iteration()) for _ in range(4)]
    orc = oracle.OracleVegas(n_dim, n)
    calls = iter(range(4))
    src = lambda m, d: oracle.uniforms_f64_philox(seed, next(calls), 0, m, d)  # noqa: E731
    ref = [orc.iteration(src, symgauss_np) for _ in range(4)]
    np.testing.assert_allclose(np.array(got), np.array(ref), rtol=RTOL)
    np.testing.assert_allclose(inst.divisions.cpu().numpy(), orc.divisions, rtol=0, atol=1e-12)


def test_fp64_breit_wigner_and_gauss_against_oracle():
    c = np.random.default_rng(3).random(5)
    cases = [(6, integrands.breit_wigner(c), lambda x: oracle.integrand_breit_wigner(x, coeffs=c)),
             (5, integrands.gauss([0.3, 0.4, 0.5, 0.6, 0.7], [0.1, 0.2, 0.05, 0.15, 0.1]),
              lambda x: oracle.integrand_gauss_mu(x, [0.3, 0.4, 0.5, 0.6, 0.7], [0.1, 0.2, 0.05, 0.15, 0.1])),
             (12, integrands.symgauss(0.2), lambda x: oracle.integrand_symgauss(x, 0.2)),
             (16, integrands.symgauss(0.3), lambda x: oracle.integrand_symgauss(x, 0.3)),
             (9, integrands.prod(), oracle.integrand_prod)]
    for n_dim, dint, ofn in cases:
        inst = VegasFlow(n_dim, 50_000, verbose=False, seed=11)
        inst.compile(dint)
        got = [tuple(float(v) for v in inst._run_iteration()) for _ in range(2)]
        orc = oracle.OracleVegas(n_dim, 50_000)
        calls = iter(range(2))
        src = lambda m, d: oracle.uniforms_f64_philox(11, next(calls), 0, m, d)  # noqa: E731
        ref = [orc.iteration(src, ofn) for _ in range(2)]
        np.testing.assert_allclose(np.array(got), np.array(ref), rtol=1e-9, err_msg=dint.__name__)


def test_fp32_injected_against_fp64_oracle():
    """The fp32 form on the float64 oracle's own uniforms: same bins (the index is
    taken in float64), the integral within a small fraction of sigma."""
    n_dim, n = 8, 1_000_000
    rng = np.random.default_rng(11)
    u = oracle.tech_cut_affine(rng.random((n, n_dim)))
    orc = oracle.OracleVegas(n_dim, n)
    ref = orc.iteration(lambda m, d: u, symgauss_np)
    inst = VegasFlow(n_dim, n, verbose=False, precision="fp32")
    inst.compile(integrands.symgauss())
    ud = dev(u)
    inst.set_uniform_source(lambda m, d: ud)
    r, s = (float(v) for v in inst._run_iteration())
    assert abs(r - ref[0]) < 0.01 * ref[1], (r, ref)
    assert abs(s - ref[1]) < 0.01 * ref[1], (s, ref)
    np.testing.assert_allclose(inst.divisions.cpu().numpy(), orc.divisions, rtol=0, atol=1e-5)


def test_c2_injected_1e7_bit_exact_indices_and_integral():
    """C2 injected mode at 1e7 events: default_rng(11) uniforms through the TECH_CUT
    affine; indices of every event bit-exact, integral to 1e-10 of the oracle."""
    n_dim, n = 8, 10_000_000
    u = oracle.tech_cut_affine(np.random.default_rng(11).random((n, n_dim)))
    ud = dev(u)
    inst = VegasFlow(n_dim, n, verbose=False)
    inst.compile(integrands.symgauss())
    x, w, ind = inst._digest_random_generation(ud)
    ox, ow, oind = oracle.vegas_map(u, oracle.initial_grid(n_dim))
    assert np.array_equal(ind.cpu().numpy(), oind)
    assert np.array_equal(x.cpu().numpy(), ox)
    assert np.array_equal(w.cpu().numpy(), ow)
    del x, w, ind
    gpu_src = chunked(ud)
    inst.set_uniform_source(gpu_src)
    r, s = (float(v) for v in inst._run_iteration())
    assert gpu_src.pos == n
    orc = oracle.OracleVegas(n_dim, n)
    ref = orc.iteration(chunked(u), symgauss_np)
    np.testing.assert_allclose([r, s], ref, rtol=1e-10)
    np.testing.assert_allclose(inst.divisions.cpu().numpy(), orc.divisions, rtol=0, atol=1e-12)


def test_c2_fp32_fused_1e8_within_sigma_of_exact():
    """C2 headline configuration: 8-D Gaussian, 1e8 events/iteration, 10
    iterations, fused fp32 form: the result is within 3 sigma of erf(5)^8."""
    inst = VegasFlow(8, 100_000_000, verbose=False, precision="fp32", seed=2)
    inst.compile(integrands.symgauss())
    res, sigma = inst.run_integration(10)
    exact = oracle.symgauss_exact(8)
    assert sigma < 1e-4
    assert abs(res - exact) < 3 * sigma, (res, sigma, exact)


def test_index_range_flag_on_bad_injected_uniforms():
    """Uniforms outside [0,1) are clamped to the grid and flagged, never read out of bounds."""
    inst = VegasFlow(2, 4, verbose=False)
    inst.compile(integrands.symgauss())
    bad = dev(np.array([[1.5, 0.5], [-0.5, 0.5], [0.5, 0.5], [0.2, 0.9]]))
    inst.set_uniform_source(lambda m, d: bad)
    inst.run_integration(1)  # logs the warning, clears the flag
    flags = inst._workspace()["flags"]
    assert int(flags[0].item()) == 0


def test_abi_rejects_bad_arguments():
    lib = nat.load()
    rc = lib.vf_sample(0, 0, None, 4, 10, 0, 0.1, None, None, 1.0, None, 1, 0, 1, None, 1, 0, None, 1,
                       None, None, None, None, None, None)
    assert rc == nat.VF_ERR_ARG
    assert b"grid" in lib.vf_last_error_string()
    rc = lib.vf_sample(0, 0, None, 17, 10, 0, 0.1, None, None, 1.0, None, 1, 0, 1, None, 1, 0, None, 1,
                       None, None, None, None, None, None)
    assert rc == nat.VF_ERR_UNSUPPORTED


@pytest.mark.parametrize("spread,empty,scale", [(1.0, 0.0, 1e-3), (4.0, 0.0, 1e-3), (8.0, 0.0, 1e-3),
                                                (2.0, 0.7, 1e-3), (2.0, 0.95, 1e-3), (2.0, 0.8, 1e12),
                                                (2.0, 0.8, 1e-40), (1.0, 1.0, 1.0)])
def test_float32_refinement_close_to_float64(spread, empty, scale):
    """vf_iteration_end with train=2 (the fp32 form's float32 refinement, its
    rebinning walk evaluated in parallel in closed form) moves the edges to
    within float32 rounding of the float64 refinement (train=1, the reference's
    sequential walk), keeps them ordered, and keeps the end points -- also for
    histograms spread over many decades, with most (or all) bins empty, and at
    scales where the reference's 1e-30 floor leaves float32's range once the
    histogram is scaled to a largest bin of 1."""
    rng = np.random.default_rng(int(spread) + int(10 * empty))
    n_dim = 6
    hist = np.exp(spread * rng.standard_normal((n_dim, 50))) * scale
    hist[rng.random((n_dim, 50)) < empty] = 0.0
    row = np.concatenate([[1.0, 1.0], hist.reshape(-1)])
    grid = np.sort(rng.random((n_dim, 51)), axis=1)
    grid[:, 0], grid[:, -1] = 0.0, 1.0
    lib = nat.load()
    out = {}
    for mode in (1, 2):
        g = dev(grid)
        part = dev(row)
        history = torch.zeros(2, dtype=torch.float64, device="cuda")
        avg = torch.zeros(5, dtype=torch.float64, device="cuda")
        nat.check(lib.vf_iteration_end(nat.ptr(part), 1, n_dim, 1, mode, 1000.0, 1.5, nat.ptr(g), None, None,
                                       nat.ptr(history), nat.ptr(avg), 0, None, nat.stream_handle()))
        out[mode] = g.cpu().numpy()
    want = np.stack([oracle.refine_grid_per_dimension(hist[d], grid[d]) for d in range(n_dim)])
    np.testing.assert_allclose(out[1], want, rtol=0, atol=1e-13)
    np.testing.assert_allclose(out[2], want, rtol=0, atol=2e-5)
    assert np.all(np.diff(out[2], axis=1) >= 0)
    assert np.all(out[2][:, 0] == 0.0) and np.all(out[2][:, -1] == 1.0)


def test_pipe_probes():
    """The calibration probes of the fused sampler's roofline run and report their
    work: FFMA chains (the issue rate) and Philox-shaped wide-multiply chains
    (the FMA-heavy pipe), the latter slower per instruction on this part."""
    import ctypes
    lib = nat.load()
    blocks = 152 * 4
    buf = torch.empty(blocks * 256, dtype=torch.float32, device="cuda")
    rates = {}
    for name in ("vf_issue_probe", "vf_widemul_probe"):
        per_thread = ctypes.c_longlong(0)
        fn = getattr(lib, name)
        nat.check(fn(nat.ptr(buf), blocks, 200, ctypes.byref(per_thread), nat.stream_handle()))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        nat.check(fn(nat.ptr(buf), blocks, 2000, ctypes.byref(per_thread), nat.stream_handle()))
        b.record()
        b.synchronize()
        assert per_thread.value == 128 * 2000
        rates[name] = blocks * 256 * per_thread.value / 32 / (a.elapsed_time(b) / 1e3)
    assert rates["vf_issue_probe"] > rates["vf_widemul_probe"] > 0
    assert lib.vf_widemul_probe(None, blocks, 10, None, None) == nat.VF_ERR_ARG


def test_bounded_device_wait_reports_timeout():
    """The TMA path's bounded mbarrier wait, on a barrier nothing completes,
    gives up and sets VF_FLAG_TIMEOUT; the context stays usable afterwards."""
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib = nat.load()
    assert lib.vf_wait_selftest(2000, nat.ptr(flag), nat.stream_handle()) == nat.VF_OK
    torch.cuda.synchronize()
    assert int(flag.item()) & nat.VF_FLAG_TIMEOUT
    inst = VegasFlow(2, 10_000, verbose=False, seed=1)
    inst.compile(integrands.symgauss())
    res, sig = inst.run_integration(2)
    assert np.isfinite(res) and sig > 0
