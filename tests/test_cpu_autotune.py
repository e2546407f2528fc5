"""Launch-shape autotuner: search space, cache keys and cache file, and the
native tunables' argument checks (no GPU needed for any of these)."""

import ctypes
import json

import pytest

from vegasflow_gb300 import VegasFlow, _native as nat, autotune


def test_launch_shape_validation():
    with pytest.raises(ValueError):
        autotune.LaunchShape(threads=64)
    with pytest.raises(ValueError):
        autotune.LaunchShape(blocks_per_sm=17)
    with pytest.raises(ValueError):
        autotune.LaunchShape(hist_copies=8)
    with pytest.raises(ValueError):
        autotune.LaunchShape(threads=256)
    s = autotune.LaunchShape(512, 1, 0)
    assert autotune.LaunchShape.from_dict(s.as_dict()) == s
    assert hash(s) == hash(autotune.LaunchShape(512, 1, 0))
    assert s != autotune.DEFAULT_SHAPE


def test_candidates_cover_the_space():
    train = autotune.candidates(train=True)
    assert len(set(train)) == len(train) == 3
    assert autotune.DEFAULT_SHAPE in train
    frozen = autotune.candidates(train=False)
    assert {c.hist_copies for c in frozen} == {0}  # no histogram when the grid is frozen
    assert autotune.DEFAULT_SHAPE in frozen


def test_events_bucket_and_key():
    assert autotune.events_bucket(10 ** 8) == autotune.events_bucket(int(1.1e8))
    assert autotune.events_bucket(10 ** 8) != autotune.events_bucket(2 * 10 ** 8)
    k1 = autotune.cache_key("GB300", 152, 0, 1, 8, 1, 10 ** 8, True)
    k2 = autotune.cache_key("GB300", 152, 0, 1, 8, 1, 10 ** 8, False)
    k3 = autotune.cache_key("GB300", 152, 0, 1, 7, 1, 10 ** 8, True)
    assert len({k1, k2, k3}) == 3


def test_cache_round_trip(tmp_path):
    path = tmp_path / "sub" / "shapes.json"
    c = autotune.TuneCache(str(path))
    assert c.get("k") is None
    c.put("k", autotune.LaunchShape(512, 1, 0), 0.5, 0.7)
    again = autotune.TuneCache(str(path))
    assert again.get("k") == autotune.LaunchShape(512, 1, 0)
    data = json.loads(path.read_text())
    assert data["k"]["ms"] == 0.5 and data["k"]["default_ms"] == 0.7


def test_cache_ignores_garbage(tmp_path):
    path = tmp_path / "shapes.json"
    path.write_text("{not json")
    assert autotune.TuneCache(str(path)).entries == {}
    path.write_text(json.dumps({"a": {"shape": {"threads": 99, "blocks_per_sm": 0, "hist_copies": 0}},
                                "b": 3}))
    c = autotune.TuneCache(str(path))
    assert c.get("a") is None and "b" not in c.entries


def test_cache_path_env(monkeypatch, tmp_path):
    monkeypatch.setenv("VEGASFLOW_GB300_TUNE_CACHE", str(tmp_path / "x.json"))
    assert autotune.cache_path() == str(tmp_path / "x.json")


def test_native_tunables_checked():
    lib = nat.load()
    v = ctypes.c_int(0)
    for key, bad in ((nat.VF_TUNE_F32_THREADS, 64), (nat.VF_TUNE_F32_THREADS, 256),
                     (nat.VF_TUNE_F32_BLOCKS_PER_SM, -1), (nat.VF_TUNE_F32_BLOCKS_PER_SM, 17),
                     (nat.VF_TUNE_F32_HIST_COPIES, 3), (nat.VF_TUNE_F32_HIST_COPIES, 8), (99, 0)):
        assert lib.vf_tune_get(key, ctypes.byref(v)) == (nat.VF_ERR_ARG if key == 99 else nat.VF_OK)
        before = v.value
        assert lib.vf_tune_set(key, bad) == nat.VF_ERR_ARG
        if key != 99:
            assert lib.vf_tune_get(key, ctypes.byref(v)) == nat.VF_OK and v.value == before
    saved = autotune.current()
    try:
        autotune.apply(autotune.LaunchShape(512, 3, 0))
        assert autotune.current() == autotune.LaunchShape(512, 3, 0)
    finally:
        autotune.apply(saved)


def test_no_shape_off_the_fused_path():
    inst = VegasFlow(2, 1000, device="cpu", precision="fp32")
    assert not autotune.fused_f32(inst)
    assert inst.launch_shape is None
