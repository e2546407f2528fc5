"""The oracle's restatements of the fp32 samplers' integer maps, pinned on the
CPU: on the uniforms the Philox words stand for, u = (word + 1/2) / 2^32, their
bins are the reference's float64 bins (``oracle.vegas_map`` / ``plus_map``, both
checked against the reference's own fixtures), and the one-rounding multiply-add
used for x is exact against rational arithmetic."""

from fractions import Fraction

import numpy as np

import oracle


def test_fma_f32_rounds_once():
    rng = np.random.default_rng(0)
    a = rng.standard_normal(4000).astype(np.float32)
    b = (1.0 + rng.random(4000)).astype(np.float32)
    c = (rng.standard_normal(4000) * 10.0 ** rng.integers(-8, 3, 4000)).astype(np.float32)
    got = oracle.fma_f32(a, b, c)
    for ai, bi, ci, gi in zip(a, b, c, got):
        exact = Fraction(float(ai)) * Fraction(float(bi)) + Fraction(float(ci))
        # the float32 neighbours of the exact value, and the nearest (ties to even)
        r = np.float32(float(exact))
        cands = [np.nextafter(r, np.float32(-np.inf)), r, np.nextafter(r, np.float32(np.inf))]
        errs = [abs(Fraction(float(v)) - exact) for v in cands]
        best = min(errs)
        winners = [v for v, e in zip(cands, errs) if e == best]
        if len(winners) == 2:
            winners = [v for v in winners if (int(np.float32(v).view(np.uint32)) & 1) == 0]
        assert gi == winners[0], (ai, bi, ci, gi, winners)


def test_vegas_f32_bins_are_the_reference_bins():
    rng = np.random.default_rng(1)
    for n_dim in (1, 3, 8, 16):
        grid = np.stack([oracle.refine_grid_per_dimension(rng.random(50) ** 3, np.linspace(0, 1, 51))
                         for _ in range(n_dim)])
        words = oracle.philox_words(77, 3, 0, 20_000, n_dim)
        # words at the ends and on every bin boundary
        edge = np.array([0, 1, 2 ** 32 - 1, 2 ** 32 - 2] + [int(k * 2 ** 32 / 50) + o for k in range(1, 50)
                                                            for o in (-1, 0, 1)], dtype=np.uint64)
        extra = np.resize(edge, (edge.size // n_dim + 1) * n_dim).reshape(-1, n_dim).astype(np.uint32)
        words = np.concatenate([words, extra])
        ind, x, w = oracle.vegas_map_f32_words(words, grid, 1.0 / words.shape[0])
        _, _, ind_ref = oracle.vegas_map(oracle.uniforms_of_words(words), grid)
        np.testing.assert_array_equal(ind, ind_ref)
        # x lies in its bin, within float32 rounding
        lo = np.take_along_axis(grid, ind.T, axis=1).T
        hi = np.take_along_axis(grid, ind.T + 1, axis=1).T
        assert np.all(x >= lo - 1e-6) and np.all(x <= hi + 1e-6)
        # the weight is the float64 weight within float32 rounding (D + 2 roundings)
        w64 = np.prod(hi - lo, axis=1) * 50.0 ** n_dim / words.shape[0]
        np.testing.assert_allclose(w, w64, rtol=(n_dim + 2) * 2.0 ** -23)


def test_vegas_f32_map_with_limits():
    """With integration limits x lies in the limits' image of its bin and the
    weight carries the box's volume, within float32 rounding."""
    rng = np.random.default_rng(4)
    n_dim = 3
    grid = np.stack([oracle.refine_grid_per_dimension(rng.random(50) ** 2, np.linspace(0, 1, 51))
                     for _ in range(n_dim)])
    xmin = np.array([-1.0, 0.25, 3.0])
    xdelta = np.array([4.0, 3.25, 0.5])
    words = oracle.philox_words(9, 2, 0, 5000, n_dim)
    ind, x, w = oracle.vegas_map_f32_words(words, grid, 1.0 / 5000, xmin, xdelta)
    ind0, _, _ = oracle.vegas_map_f32_words(words, grid, 1.0 / 5000)
    np.testing.assert_array_equal(ind, ind0)  # the bins do not depend on the limits
    lo = xmin + np.take_along_axis(grid, ind.T, axis=1).T * xdelta
    hi = xmin + np.take_along_axis(grid, ind.T + 1, axis=1).T * xdelta
    assert np.all(x >= lo - 1e-5) and np.all(x <= hi + 1e-5)
    w64 = np.prod((hi - lo), axis=1) * 50.0 ** n_dim / 5000
    np.testing.assert_allclose(w, w64, rtol=(n_dim + 4) * 2.0 ** -23)


def test_f32_weight_prescale_keeps_16d_weights_in_range():
    """Narrow bins at 16 dimensions: prod_d delta underflows float32 without the
    power-of-two prescale, with it the weight keeps float32 precision."""
    n_dim = 16
    edges = np.concatenate([[0.0], np.linspace(0.001, 1.0, 50)])  # bin 0 is 0.001 wide
    grid = np.tile(edges, (n_dim, 1))
    words = np.full((4, n_dim), 0xFFFFFFFF, dtype=np.uint32)  # u -> 1: bin 0 in every dimension
    ind, _, w = oracle.vegas_map_f32_words(words, grid, 1.0)
    assert np.all(ind == 0)
    w64 = 0.001 ** n_dim * 50.0 ** n_dim
    assert np.float32(0.001) ** n_dim == 0.0  # the plain float32 product underflows
    np.testing.assert_allclose(w, w64, rtol=18 * 2.0 ** -23)


def test_plus_f32_bins_are_the_reference_bins():
    rng = np.random.default_rng(2)
    for n_dim, n_strat in ((2, 70), (3, 21), (6, 4), (4, 10), (1, 9999)):
        n_hcubes = min(n_strat ** n_dim, 400)
        n_ev = rng.integers(2, 30, n_hcubes).astype(np.int32)
        n = int(n_ev.sum())
        words = oracle.philox_words(5, 1, 0, n, n_dim)
        h = np.repeat(np.arange(n_hcubes), n_ev)
        points = oracle.hypercube_points(n_hcubes, n_strat, n_dim)[h]
        got = oracle.plus_bins_from_words(words, points, n_strat)
        grid = oracle.initial_grid(n_dim)
        _, _, ind_ref, _ = oracle.plus_map(oracle.uniforms_of_words(words), n_strat, n_ev, grid)
        np.testing.assert_array_equal(got, ind_ref)
