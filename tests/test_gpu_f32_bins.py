"""Bin-index parity of the fp32 kernels that earn the benchmark numbers.

The fused fp32 VEGAS sampler, its TMA injected-uniform path and the fp32
VEGAS+ sampler each have a parity instantiation that writes every event's bin
indices (reached through ``vf_sample`` / ``vf_plus_sample`` with ``ind_out`` as
the only tap).  On the same Philox words the indices must equal the
reference's float64 bins of the uniforms the words stand for,
u = (word + 1/2) / 2^32 (``oracle.vegas_map`` / ``oracle.plus_map``, restating
vflow.py:93-126, :67 and vflowplus.py:46-80, both pinned to the reference's
own fixtures), and for injected float64 uniforms the reference's bins of those
uniforms.  Bar: ``assert_array_equal`` on every index.  The map kernel of the
sampler API (the same draw without an integrand) is also checked for its
points and weights, bit for bit against the oracle's restatement, with and
without integration limits."""

import numpy as np
import pytest
import torch

import oracle
from vegasflow_gb300 import VegasFlow, VegasFlowPlus, integrands
from vegasflow_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def _trained(n_dim, n, integrand, seed=31, iters=3, **limits):
    inst = VegasFlow(n_dim, n, verbose=False, precision="fp32", seed=seed, **limits)
    inst.compile(integrand)
    inst.run_integration(iters)
    return inst


def _reference_bins(u, grid, chunk=1_000_000):
    out = np.empty(u.shape, dtype=np.int32)
    for s in range(0, u.shape[0], chunk):
        _, _, out[s:s + chunk] = oracle.vegas_map(u[s:s + chunk], grid)
    return out


@pytest.mark.parametrize("n_dim", [1, 3, 8, 16])
@pytest.mark.parametrize("which", ["symgauss", "prod"])
@pytest.mark.parametrize("offset", [0, (1 << 32) - 300_000])
def test_fused_sampler_bins_are_the_reference_bins(n_dim, which, offset):
    """Philox path: D = 1, 3 take the two-events-per-pass loop, D = 8, 16 the
    single one; an event offset near 2^32 makes the counter's high word change
    inside the launch."""
    n, call = 1_000_000, 7
    f = integrands.symgauss(0.2) if which == "symgauss" else integrands.prod()
    inst = _trained(n_dim, n, f)
    ind = torch.full((n, n_dim), -1, dtype=torch.int32, device="cuda")
    inst._sample(n, offset, call, inst._int_id, inst._params_dev, True, False, ind=ind)
    torch.cuda.synchronize()
    words = oracle.philox_words(inst._seed, call, offset, n, n_dim)
    want = _reference_bins(oracle.uniforms_of_words(words), inst.divisions.cpu().numpy())
    np.testing.assert_array_equal(ind.cpu().numpy(), want)


@pytest.mark.parametrize("n_dim,offset", [(1, 0), (3, 0), (5, 0), (8, 0), (16, 0), (8, (1 << 32) - 300_000)])
@pytest.mark.parametrize("with_ind", [True, False])
def test_map_kernel_points_and_weights_match_oracle(n_dim, offset, with_ind):
    """x, w (and bins) of the map kernel bit for bit against the oracle's
    restatement; n is not a multiple of the warp tiles, so the last tile takes
    the plain-store path; an event offset near 2^32 makes the counter's high
    word change inside the launch."""
    n, call = 1_000_003, 5
    inst = _trained(n_dim, n, integrands.symgauss(0.2))
    x = torch.empty((n, n_dim), dtype=torch.float32, device="cuda")
    w = torch.empty(n, dtype=torch.float32, device="cuda")
    ind = torch.empty((n, n_dim), dtype=torch.int32, device="cuda") if with_ind else None
    inst._sample(n, offset, call, nat.VF_INT_NONE, None, False, False, ind=ind, x=x, w=w)
    torch.cuda.synchronize()
    words = oracle.philox_words(inst._seed, call, offset, n, n_dim)
    grid = inst.divisions.cpu().numpy()
    ind_o, x_o, w_o = oracle.vegas_map_f32_words(words, grid, inst.xjac)
    if with_ind:
        np.testing.assert_array_equal(ind.cpu().numpy(), ind_o)
    np.testing.assert_array_equal(ind_o, _reference_bins(oracle.uniforms_of_words(words), grid))
    np.testing.assert_array_equal(x.cpu().numpy().view(np.uint32), x_o.view(np.uint32))
    np.testing.assert_array_equal(w.cpu().numpy().view(np.uint32), w_o.view(np.uint32))


@pytest.mark.parametrize("n_dim", [3, 8])
def test_map_kernel_with_limits_matches_oracle(n_dim):
    """Integration limits fold into the table (c0 = fma(lo - delta, xdelta, xmin),
    c1 = delta xdelta): x in the limits' box and w with its volume, bit for bit."""
    n, call = 500_003, 6
    rng = np.random.default_rng(n_dim)
    xmin = rng.uniform(-2.0, 1.0, n_dim)
    xmax = xmin + rng.uniform(0.1, 4.0, n_dim)
    inst = _trained(n_dim, n, integrands.prod(), xmin=list(xmin), xmax=list(xmax))
    x = torch.empty((n, n_dim), dtype=torch.float32, device="cuda")
    w = torch.empty(n, dtype=torch.float32, device="cuda")
    inst._sample(n, 0, call, nat.VF_INT_NONE, None, False, False, x=x, w=w)
    torch.cuda.synchronize()
    words = oracle.philox_words(inst._seed, call, 0, n, n_dim)
    grid = inst.divisions.cpu().numpy()
    _, x_o, w_o = oracle.vegas_map_f32_words(words, grid, inst.xjac, inst._xmin_np, inst._xdelta_np)
    np.testing.assert_array_equal(x.cpu().numpy().view(np.uint32), x_o.view(np.uint32))
    np.testing.assert_array_equal(w.cpu().numpy().view(np.uint32), w_o.view(np.uint32))


def _near_edge_uniforms(n_dim):
    """Uniforms a few float64 ulps around every bin edge 1 - k/50 (k = 1..49)
    and near the ends of the reference's range [1e-8, 1 - 1e-8)."""
    vals = []
    for k in range(1, 50):
        x = y = 1.0 - k / 50.0
        vals.append(x)
        for _ in range(40):
            x = np.nextafter(x, 2.0)
            y = np.nextafter(y, -1.0)
            vals += [x, y]
    vals += [1e-8, np.nextafter(1e-8, 1.0), 1.0 - 1e-8, np.nextafter(1.0 - 1e-8, 0.0), 2.0 ** -12,
             np.nextafter(2.0 ** -12, 0.0), 2.0 ** -13]
    vals = np.array(vals)
    rows = (vals.size + n_dim - 1) // n_dim
    return np.resize(vals, rows * n_dim).reshape(rows, n_dim)


@pytest.mark.parametrize("n_dim,n,misalign", [(8, 10_000_000, False), (16, 1_000_000, False),
                                              (4, 1_000_000, False), (8, 1_000_000, True),
                                              (5, 1_000_000, False), (1, 300_000, False),
                                              (2, 300_000, False), (12, 1_000_000, False)])
def test_injected_fused_bins_are_the_reference_bins(n_dim, n, misalign):
    """C2's injected mode (default_rng(11) through the TECH_CUT affine) with the
    near-edge uniforms first: the TMA path (D = 4, 8, 16 on an aligned array)
    and the plain-load path (misaligned, or D = 5)."""
    u = oracle.tech_cut_affine(np.random.default_rng(11).random((n, n_dim)))
    edge = _near_edge_uniforms(n_dim)
    u[:edge.shape[0]] = edge
    inst = _trained(n_dim, n, integrands.symgauss(0.2), iters=2)
    if misalign:
        buf = torch.empty(n * n_dim + 1, dtype=torch.float64, device="cuda")
        ud = buf[1:].view(n, n_dim)
        ud.copy_(torch.as_tensor(u, device="cuda"))
        assert ud.data_ptr() % 16 == 8
    else:
        ud = torch.as_tensor(u, device="cuda").contiguous()
        assert ud.data_ptr() % 16 == 0
    ind = torch.full((n, n_dim), -1, dtype=torch.int32, device="cuda")
    ws = inst._workspace()
    ws["flags"].zero_()
    inst._sample(n, 0, 0, inst._int_id, inst._params_dev, True, False, u_inj=ud, ind=ind)
    torch.cuda.synchronize()
    assert int(ws["flags"][0].item()) == 0
    np.testing.assert_array_equal(ind.cpu().numpy(), _reference_bins(u, inst.divisions.cpu().numpy()))


@pytest.mark.parametrize("n_dim,n_events,adaptive,which", [(6, 2_000_000, True, "bw"),
                                                           (3, 200_000, False, "symgauss"),
                                                           (2, 100_000, True, "symgauss"),
                                                           (9, 300_000, False, "bw")])
def test_plus_fp32_bins_are_the_reference_bins(n_dim, n_events, adaptive, which):
    """The fp32 VEGAS+ sampler's integer stratified map on a trained grid and a
    reallocated event layout (C3: 6-D Breit-Wigner, adaptive, 2e6 events)."""
    if which == "bw":
        f = integrands.breit_wigner(np.random.default_rng(3).random(n_dim - 1))
    else:
        f = integrands.symgauss(0.2)
    inst = VegasFlowPlus(n_dim, n_events, adaptive=adaptive, verbose=False, precision="fp32", seed=13)
    inst.compile(f)
    inst.run_integration(2)
    n_total = int(inst.n_events)
    n_ev = inst.n_ev.cpu().numpy()
    assert int(n_ev.sum()) == n_total
    ind = torch.full((n_total, n_dim), -1, dtype=torch.int32, device="cuda")
    x = torch.empty((n_total, n_dim), dtype=torch.float32, device="cuda")
    ws = inst._plus_buffers()
    call = 9
    nat.call("vf_plus_sample", nat.VF_PREC_F32, nat.ptr(inst.divisions), n_dim, inst._n_strat, inst._n_hcubes,
             nat.ptr(inst.n_ev), nat.ptr(inst._ev_start), float(inst.xjac), None, None, 1.0, None, inst._seed,
             call, inst._int_id, nat.ptr(inst._params_dev), 0, nat.ptr(ws["ress"]), nat.ptr(ws["ress2"]),
             nat.ptr(ws["partials"]), inst._rows, nat.ptr(ind), nat.ptr(x), None, None, nat.stream_handle())
    torch.cuda.synchronize()
    words = oracle.philox_words(inst._seed, call, 0, n_total, n_dim)
    grid = inst.divisions.cpu().numpy()
    x64, _, want, _ = oracle.plus_map(oracle.uniforms_of_words(words), inst._n_strat, n_ev, grid)
    got = ind.cpu().numpy()
    np.testing.assert_array_equal(got, want)
    h = np.repeat(np.arange(inst._n_hcubes), n_ev)
    pts = oracle.hypercube_points(inst._n_hcubes, inst._n_strat, n_dim)[h]
    np.testing.assert_array_equal(got, oracle.plus_bins_from_words(words, pts, inst._n_strat))
    # the points: bit for bit against the oracle's float32 restatement, and within
    # 2e-6 of the float64 map
    xg = x.cpu().numpy()
    np.testing.assert_array_equal(xg.view(np.uint32),
                                  oracle.plus_map_f32_words(words, pts, inst._n_strat, grid).view(np.uint32))
    assert np.max(np.abs(xg.astype(np.float64) - x64)) < 2e-6


@pytest.mark.parametrize("n_dim,call,offset", [(1, 0, 0), (8, 3, 5), (11, (1 << 28) + 2, 1 << 33)])
def test_philox_uniforms_are_the_words_uniforms(n_dim, call, offset):
    """vf_philox_uniforms writes u = (word + 1/2) / 2^32 of the samplers' words."""
    n, seed = 100_000, 77
    u = torch.empty((n, n_dim), dtype=torch.float64, device="cuda")
    nat.call("vf_philox_uniforms", seed, call, call >> 28, offset, n, n_dim, nat.ptr(u), nat.stream_handle())
    torch.cuda.synchronize()
    want = oracle.uniforms_of_words(oracle.philox_words(seed, call, offset, n, n_dim))
    np.testing.assert_array_equal(u.cpu().numpy(), want)
