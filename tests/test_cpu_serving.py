"""Host-side logic of the serving loop and the batch engine (no GPU)."""

import numpy as np

from vegasflow_gb300 import integrands
from vegasflow_gb300.batch import ITEM_DTYPE, c4_specs
from vegasflow_gb300.serving import (SERVE_TILE_MIN, launch_groups, percentile, poisson_workload, request_footprint,
                                     serving_tile_events, step_tables)


def test_step_tables_cover_every_event():
    n_events = [10, 65536, 65537, 300_000, 1]
    n_dim = [2, 8, 16, 3, 1]
    t = step_tables(n_events, n_dim, slots=[4, 0, 7, 2, 9], stream_ids=[1, 2, 3, 4, 5],
                    integrand_ids=[1, 2, 2, 3, 4], grid_off=[0, 1, 2, 3, 4], param_off=[0, 1, 2, 3, 4],
                    tile_events=65536)
    items = t["items"]
    assert items.dtype == ITEM_DTYPE and list(items["slot"]) == [4, 0, 7, 2, 9]
    for i, (n, d) in enumerate(zip(n_events, n_dim)):
        sel = t["tile_item"] == i
        assert items["n_tiles"][i] == sel.sum() == -(-n // 65536)
        assert items["tile0"][i] == np.flatnonzero(sel)[0]
        assert t["tile_count"][sel].sum() == n
        np.testing.assert_array_equal(t["tile_start"][sel], np.arange(sel.sum()) * 65536)
        # iteration-end blocks: one per dimension and one for the sums
        roles = t["blk_role"][t["blk_item"] == i]
        np.testing.assert_array_equal(roles, list(range(d)) + [-1])
    widths = 2 + 50 * np.repeat(n_dim, items["n_tiles"])
    np.testing.assert_array_equal(np.diff(t["tile_row"]), widths[:-1])
    assert t["rows_total"] == widths.sum()


def test_served_tile_sizes():
    """About 512 tiles per request, multiples of 256 events, between 2,048 and
    65,536 events; tables with one tile size per request cover every event."""
    n_events = np.array([1, 10_000, 1_000_000, 2_000_000, 10_000_000, 10 ** 9])
    t = serving_tile_events(n_events)
    assert np.all(t % 256 == 0) and np.all(t >= SERVE_TILE_MIN) and np.all(t <= 65536)
    np.testing.assert_array_equal(t, [2048, 2048, 2048, 4096, 19712, 65536])
    assert np.all((n_events + t - 1) // t <= np.maximum(512, n_events // 65536 + 1))
    n_dim = [3, 8, 16, 6, 12, 2]
    tab = step_tables(n_events[:5], n_dim[:5], slots=range(5), stream_ids=range(5), integrand_ids=[1] * 5,
                      grid_off=range(5), param_off=range(5), tile_events=t[:5])
    for i, (n, size) in enumerate(zip(n_events[:5], t[:5])):
        sel = tab["tile_item"] == i
        assert tab["items"]["n_tiles"][i] == sel.sum() == -(-n // size)
        assert tab["tile_count"][sel].sum() == n and tab["tile_count"][sel].max() <= size
        np.testing.assert_array_equal(tab["tile_start"][sel], np.arange(sel.sum()) * size)


def test_step_tables_of_no_requests():
    t = step_tables([], [], [], [], [], [], [], serving_tile_events([]))
    assert t["n_tiles"] == 0 and t["rows_total"] == 0 and t["items"].size == 0
    assert t["tile_item"].size == t["tile_row"].size == t["blk_item"].size == 0


def test_footprint_grows_with_tiles():
    a = request_footprint(8, 10_000)
    b = request_footprint(8, 10_000_000)
    assert 0 < a < b and b < 1e8


def test_poisson_workload_statistics():
    reqs = poisson_workload(rate=200.0, duration=60.0, seed=9)
    assert 11_000 < len(reqs) < 13_000
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0) and arr[-1] <= 60.0
    bw = np.mean([r.integrand.__name__ == "breit_wigner" for r in reqs])
    assert 0.17 < bw < 0.23
    dims = [r.n_dim for r in reqs if r.integrand.__name__ == "gauss"]
    assert min(dims) == 2 and max(dims) == 16
    assert all(r.target_rel_sigma == 1e-3 and r.max_iterations == 20 for r in reqs)


def test_percentile_and_c4_specs():
    assert percentile([1, 2, 3, 4], 50) == 2.5
    specs = c4_specs()
    assert len(specs) == 1024
    assert all(2 <= d <= 16 and 10_000 <= n <= 10_000_000 for d, n, _ in specs)
    assert all(isinstance(f, integrands.DeviceIntegrand) for _, _, f in specs)


def test_launch_groups():
    """One sampler launch per run of (program, dimension class); the built-in
    classes share one launch when either is smaller than the persistent grid."""
    from types import SimpleNamespace as R

    act = [R(program=0, n_dim=4), R(program=0, n_dim=6), R(program=0, n_dim=12), R(program=1001, n_dim=3),
           R(program=1002, n_dim=9), R(program=1002, n_dim=16)]
    tiles = [10, 5, 400, 7, 3, 2]
    assert launch_groups(act, tiles, 10) == [(0, 15, 8, None), (15, 400, 16, None), (415, 7, 8, 1001),
                                             (422, 5, 16, 1002)]
    assert launch_groups(act, tiles, 100) == [(0, 415, 16, None), (415, 7, 8, 1001), (422, 5, 16, 1002)]
    assert launch_groups(act[3:], tiles[3:], 100) == [(0, 7, 8, 1001), (7, 5, 16, 1002)]
    assert launch_groups([], [], 100) == []
