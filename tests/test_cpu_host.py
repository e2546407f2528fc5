"""Host-side logic that needs no GPU: constructor validation, grid JSON I/O,
configuration, and the refusal to compute without CUDA (no CPU fallback)."""

import json

import numpy as np
import pytest
import torch

import oracle
from vegasflow_gb300 import PlainFlow, VegasFlow, configflow, float_me, int_me, integrands


def test_integration_limits_checks():
    """test_misc.py:85-97."""
    with pytest.raises(ValueError):
        PlainFlow(1, 10, xmin=[10], xmax=[1], device="cpu")
    with pytest.raises(ValueError):
        PlainFlow(1, 10, xmin=[10], device="cpu")
    with pytest.raises(ValueError):
        PlainFlow(1, 10, xmax=[10], device="cpu")
    with pytest.raises(ValueError):
        PlainFlow(2, 10, xmin=[0], xmax=[1], device="cpu")
    with pytest.raises(ValueError):
        PlainFlow(2, 10, xmin=[0, 1], xmax=[1], device="cpu")


def test_dimension_and_precision_validation():
    with pytest.raises(ValueError):
        VegasFlow(17, 100, device="cpu")
    with pytest.raises(ValueError):
        VegasFlow(0, 100, device="cpu")
    with pytest.raises(ValueError):
        VegasFlow(2, 100, precision="fp16", device="cpu")


def test_initial_grid_matches_reference():
    inst = VegasFlow(3, 100, device="cpu")
    np.testing.assert_array_equal(inst.divisions.numpy(), oracle.initial_grid(3))
    assert inst.grid_bins == 51


def test_save_and_load_grid_json(tmp_path):
    """test_algs.py:102-148 on the host side: JSON round trip and the errors."""
    inst = VegasFlow(2, 100, device="cpu")
    grid = np.sort(np.random.default_rng(0).random((2, 51)), axis=1)
    inst.load_grid(numpy_grid=grid)
    np.testing.assert_array_equal(inst.divisions.numpy(), grid)
    fname = tmp_path / "grid.json"
    inst.save_grid(str(fname))
    d = json.load(open(fname))
    assert set(d) == {"dimensions", "ALPHA", "BINS", "integrand", "grid"}
    assert d["dimensions"] == 2 and d["BINS"] == 51 and d["ALPHA"] == 1.5
    np.testing.assert_array_equal(np.array(d["grid"]), grid)
    other = VegasFlow(2, 100, device="cpu")
    other.load_grid(file_name=str(fname))
    np.testing.assert_array_equal(other.divisions.numpy(), grid)
    jdict = {"grid": grid.tolist(), "BINS": 0}
    json.dump(jdict, open(fname, "w"))
    with pytest.raises(ValueError):
        other.load_grid(file_name=str(fname))
    jdict["dimensions"] = -4
    json.dump(jdict, open(fname, "w"))
    with pytest.raises(ValueError):
        other.load_grid(file_name=str(fname))
    with pytest.raises(ValueError):
        other.load_grid(file_name=str(fname), numpy_grid=grid)
    with pytest.raises(ValueError):
        other.load_grid()


def test_no_cpu_fallback():
    inst = VegasFlow(2, 1000, device="cpu", verbose=False)
    inst.compile(integrands.symgauss())
    with pytest.raises(RuntimeError, match="CUDA"):
        inst.run_integration(1)


def test_compile_requires_callable():
    inst = VegasFlow(2, 100, device="cpu")
    with pytest.raises(TypeError):
        inst.compile(42)


def test_run_before_compile_raises():
    inst = PlainFlow(2, 100, device="cpu")
    with pytest.raises(RuntimeError):
        inst._recompile()


def test_casts_and_dtypes():
    """test_config.py:11-19."""
    assert int_me(4).dtype == configflow.DTYPEINT
    assert float_me(4.0).dtype == configflow.DTYPE
    assert configflow.DTYPE == torch.float64 and configflow.DTYPEINT == torch.int32


def test_float_env(monkeypatch):
    """test_config.py:22-53: VEGASFLOW_FLOAT / VEGASFLOW_INT select the dtypes."""
    import importlib
    monkeypatch.setenv("VEGASFLOW_FLOAT", "32")
    monkeypatch.setenv("VEGASFLOW_INT", "64")
    mod = importlib.reload(configflow)
    try:
        assert mod.DTYPE == torch.float32 and mod.DTYPEINT == torch.int64
        assert mod.DEFAULT_PRECISION == "fp32"
    finally:
        monkeypatch.delenv("VEGASFLOW_FLOAT")
        monkeypatch.delenv("VEGASFLOW_INT")
        importlib.reload(configflow)


def test_integrand_params():
    p = integrands.symgauss(0.1).params(4)
    assert p[0] == 0.1 and abs(p[1] - (1 / 0.1 / np.sqrt(np.pi)) ** 4) < 1e-9
    g = integrands.gauss([0.4, 0.6], [0.1, 0.2])
    np.testing.assert_array_equal(g.params(2), [0.4, 0.6, 0.1, 0.2])
    with pytest.raises(ValueError):
        g.check_dims(3)
    bw = integrands.breit_wigner([0.1, 0.2, 0.3])
    np.testing.assert_array_equal(bw.params(4), [91.19, 2.5, 0.1, 0.2, 0.3])
    with pytest.raises(ValueError):
        bw.params(6)


def test_integrand_torch_forms_match_oracle():
    x = np.random.default_rng(1).random((100, 3))
    t = torch.as_tensor(x)
    np.testing.assert_allclose(integrands.symgauss(0.1)(t).numpy(), oracle.integrand_symgauss(x, 0.1),
                               rtol=1e-13)
    c = [0.3, 0.7]
    np.testing.assert_allclose(integrands.breit_wigner(c)(t).numpy(),
                               oracle.integrand_breit_wigner(x, coeffs=c), rtol=1e-13)
    np.testing.assert_allclose(integrands.prod()(t).numpy(), oracle.integrand_prod(x), rtol=1e-15)


def test_plus_stratification_matches_reference(golden):
    """vflowplus.py:105-139 (float32 powers) against the reference's own values."""
    from vegasflow_gb300.vflowplus import stratification

    for row in golden["strat/table"]:
        n_dim, n_ev, adapt, adapt_eff, n_strat, n_h, min_neval, n_events = (int(v) for v in row)
        assert stratification(n_dim, n_ev, bool(adapt)) == (bool(adapt_eff), n_strat, n_h, min_neval,
                                                            n_events), row


def test_plus_host_state():
    from vegasflow_gb300 import VegasFlowPlus

    inst = VegasFlowPlus(6, 2_000_000, adaptive=True, device="cpu")
    assert inst.n_hypercubes == 4096 and inst.min_neval_hcube == 244 and inst.n_events == 999_424
    assert inst.xjac == 1.0 / 4096
    assert int(inst._ev_start[-1]) == inst.n_events and inst._ev_start[1] == 244
    assert inst._events_limit == 2_000_000
    inst2 = VegasFlowPlus(14, 100_000, adaptive=True, device="cpu")
    assert inst2._adaptive is False and inst2.n_hypercubes == 1


CAMEL_SRC = """
__device__ vf_real camel(const vf_real* x, int n_dim, vf_real weight, const double* params) {
  vf_real s1 = 0, s2 = 0;
  for (int d = 0; d < n_dim; ++d) {
    const vf_real t1 = (x[d] - (vf_real)params[0]) / (vf_real)params[2];
    const vf_real t2 = (x[d] - (vf_real)params[1]) / (vf_real)params[2];
    s1 += t1 * t1;
    s2 += t2 * t2;
  }
  return exp(-s1) + exp(-s2);
}
"""


def test_cuda_integrand_compiles_without_gpu():
    """NVRTC compiles the user source with the sampler on the host."""
    f = integrands.cuda_integrand(CAMEL_SRC, "camel", params=[0.3, 0.7, 0.1])
    for alg, prec in ((0, 1), (0, 0), (1, 1), (1, 0), (2, 1), (2, 0), (3, 1)):
        ok, log = f.check(alg, prec, 5)
        assert ok, log
    ok, _ = f.check(3, 0, 5)  # the batched sampler is fp32 only
    assert not ok
    bad = integrands.cuda_integrand("__device__ vf_real bad(const vf_real* x) { return y; }", "bad")
    ok, log = bad.check()
    assert not ok and "undefined" in log


def test_generate_condition_function():
    """test_utils.py:40-70: 'and', 'or', a list of conditions, and the errors."""
    from vegasflow_gb300.utils import generate_condition_function

    rng = np.random.default_rng(2)
    np_masks = rng.integers(2, size=(4, 15)).astype(bool)
    masks = [torch.as_tensor(m) for m in np_masks]

    def check(np_mask, mask, idx):
        np.testing.assert_array_equal(np_mask, mask.numpy())
        np.testing.assert_array_equal(np.array(np_mask.nonzero()).T, idx.numpy())
        assert idx.dtype == torch.int32

    check(np.all(np_masks, axis=0), *generate_condition_function(4, "and")(*masks))
    check(np.any(np_masks, axis=0), *generate_condition_function(4, "or")(*masks))
    check(np_masks[0] & np_masks[1] | np_masks[2], *generate_condition_function(3, ["and", "or"])(*masks[:3]))
    for args in ((1, "and"), (5, "bad_condition"), (5, ["or", "and"]), (3, ["or", "bad_condition"])):
        with pytest.raises(ValueError):
            generate_condition_function(*args)


def test_state_buffer_layout():
    """Average, flags word and history rows share one float64 buffer (one D2H copy
    per run_integration); growing the history keeps what is there."""
    inst = VegasFlow(2, 100, verbose=False, device="cpu")
    ws = inst._workspace()
    state = ws["state"]
    assert ws["avg"].data_ptr() == state.data_ptr()
    assert ws["flags"].dtype == torch.int32 and ws["flags"].numel() == 2
    assert ws["flags"].data_ptr() == state[5:6].data_ptr()
    assert ws["history"].data_ptr() == state[6:].data_ptr() and tuple(ws["history"].shape) == (16, 2)
    ws["avg"][:] = torch.arange(5, dtype=torch.float64)
    ws["flags"][0] = 4
    ws["history"][3] = torch.tensor([1.5, 0.25], dtype=torch.float64)
    host = state[: 5 + 1 + 4 * 2].numpy()
    assert int(host[5:6].view(np.int32)[0]) == 4
    np.testing.assert_array_equal(host[6:].reshape(4, 2)[3], [1.5, 0.25])
    inst._state_rows(ws, 64)
    assert tuple(ws["history"].shape) == (64, 2)
    np.testing.assert_array_equal(ws["avg"].numpy(), np.arange(5.0))
    assert int(ws["flags"][0]) == 4
    np.testing.assert_array_equal(ws["history"][3].numpy(), [1.5, 0.25])


@pytest.mark.parametrize("name", ["f", "x", "w", "p"])
def test_cuda_integrand_any_function_name(name):
    """A user function may be named like a sampler local (f, x, w, ...): the
    samplers reach it through a global-scope wrapper."""
    src = (f"__device__ vf_real {name}(const vf_real* y, int n_dim, vf_real weight, const double* q) "
           "{ vf_real r = 1; for (int d = 0; d < n_dim; ++d) r *= y[d]; return r; }")
    f = integrands.cuda_integrand(src, name)
    for alg, prec in ((0, 1), (0, 0), (2, 1), (3, 1)):
        ok, log = f.check(alg, prec, 3)
        assert ok, (name, alg, prec, log)
