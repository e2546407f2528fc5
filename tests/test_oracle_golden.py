"""The oracle against fixtures produced by the reference vegasflow itself.

``tests/golden/make_golden.py`` ran the reference's unmodified modules on
injected uniforms; these tests replay the same uniforms through ``oracle`` and
require: bin indices, points and weights bit-exact; integrals, sigmas, the
per-bin histogram and the refined grids equal to 1e-12 relative (reduction order
is the only freedom)."""

import numpy as np
import pytest

import oracle
from conftest import raw_blocks, replay_source

RTOL = 1e-12


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors of the published algorithm (Random123)."""
    kat = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
           ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
           ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
            (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, want in kat:
        got = [int(v) for v in oracle.philox4x32_10(ctr, key)]
        assert got == list(want)


def test_refine_matches_reference(golden):
    for t_res, sub, want in zip(golden["refine/in"], golden["refine/sub"], golden["refine/out"]):
        got, flag = oracle.refine_grid_per_dimension(t_res, sub, return_flag=True)
        assert flag == 0
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=1e-15)
        assert got[0] == 0.0 and got[-1] == 1.0
        assert np.all(np.diff(got) >= 0)


def test_map_bit_exact(golden):
    x, w, ind = oracle.vegas_map(golden["map/rnds"], golden["map/grid"])
    np.testing.assert_array_equal(ind, golden["map/ind"])
    np.testing.assert_array_equal(x, golden["map/x"])
    np.testing.assert_array_equal(w, golden["map/w"])


def test_consume_array_into_indices(golden):
    got = oracle.consume_array_into_indices(golden["consume/in"], golden["consume/idx"], 50)
    np.testing.assert_allclose(got, golden["consume/out"], rtol=RTOL)
    # the reference test's own check: a Python loop (test_utils.py:11-30)
    loop = np.zeros(50)
    for v, i in zip(golden["consume/in"], golden["consume/idx"]):
        loop[i] += v
    np.testing.assert_allclose(got, loop, rtol=RTOL)


def _symgauss(x):
    return oracle.integrand_symgauss(x, 0.1)


def _quirky(x):
    n_dim = x.shape[1]
    n100 = 100.0 * n_dim
    coef = np.sum(np.arange(n100 + 1))
    t = (x - 0.5) / 0.1
    coef = coef + np.sum(t * t, axis=1)
    coef = coef - (n100 + 1) * n100 / 2.0
    return (1.0 / 0.1 / np.sqrt(np.pi)) ** n_dim * np.exp(-coef)


CASES = {
    "vegas4": (lambda g: oracle.OracleVegas(4, 2000), _symgauss, 3, None),
    "vegas4_chunks": (lambda g: oracle.OracleVegas(4, 1500, events_limit=400), _symgauss, 2, None),
    "vegas2_quirky": (lambda g: oracle.OracleVegas(2, 1000), _quirky, 3, None),
    "vegas_limits": (lambda g: oracle.OracleVegas(3, 1200, xmin=g["vegas_limits/xmin"],
                                                  xmax=g["vegas_limits/xmax"]),
                     oracle.integrand_prod, 2, None),
    "vegas_freeze": (lambda g: oracle.OracleVegas(3, 1000), _symgauss, 3, 2),
    "plain3": (lambda g: oracle.OraclePlain(3, 1500), _symgauss, 2, None),
    "plus2": (lambda g: oracle.OraclePlus(2, 2000, adaptive=False), _symgauss, 2, None),
    "plus3_adaptive": (lambda g: oracle.OraclePlus(3, 4000, adaptive=True), _symgauss, 3, None),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_integration_replay(golden, name):
    make, integrand, n_iter, freeze_after = CASES[name]
    inst = make(golden)
    source = replay_source(raw_blocks(golden, name), oracle.tech_cut_affine)
    grids, n_evs = [], []
    for it in range(n_iter):
        if freeze_after is not None and it == freeze_after:
            inst.train = False
        if hasattr(inst, "n_ev"):
            n_evs.append(inst.n_ev.copy())
        inst.history.append(inst.iteration(source, integrand))
        if hasattr(inst, "divisions"):
            grids.append(inst.divisions.copy())
            if it == 0:
                t = inst.last["taps"][0]
                np.testing.assert_array_equal(t["ind"], golden[f"{name}/ind0"])
                np.testing.assert_array_equal(t["x"], golden[f"{name}/x0"])
                np.testing.assert_array_equal(t["w"], golden[f"{name}/w0"])
                if f"{name}/arr_res2_0" in golden.files and inst.train and len(inst.last["taps"]) == 1:
                    np.testing.assert_allclose(inst.last["arr_res2"], golden[f"{name}/arr_res2_0"],
                                               rtol=RTOL)
    np.testing.assert_allclose(np.array(inst.history), golden[f"{name}/history"], rtol=RTOL)
    final = oracle.weighted_average(inst.history)
    np.testing.assert_allclose(final, golden[f"{name}/final"], rtol=RTOL)
    if grids:
        np.testing.assert_allclose(np.stack(grids), golden[f"{name}/grids"], rtol=RTOL, atol=1e-15)
    if n_evs:
        np.testing.assert_array_equal(np.stack(n_evs), golden[f"{name}/n_ev"])


def test_plus_stratification_table(golden):
    for row in golden["strat/table"]:
        n_dim, n_ev, adapt, adapt_eff, n_strat, n_h, min_neval, n_events = (int(v) for v in row)
        got = oracle.plus_stratification(n_dim, n_ev, bool(adapt))
        assert got == (bool(adapt_eff), n_strat, n_h, min_neval, n_events), row


def test_exact_integrals():
    assert abs(oracle.symgauss_exact(4) - 0.99999999999385) < 1e-13
    assert abs(oracle.symgauss_exact(8) - 0.99999999998770) < 1e-13
    c = np.random.default_rng(3).random(5)
    bw = oracle.breit_wigner_exact(6, coeffs=c)
    assert abs(bw / np.prod(1 + c / 2) - 0.0135380693) < 1e-9
