"""Launch-shape autotuner for the fused fp32 VEGAS sampler.

The sampler's speed depends on three choices that do not change its results
beyond float rounding (the Philox stream is indexed by event, not by thread):

* ``threads``       -- block size, 1024 or 512 (one or two resident blocks per
  SM at 64 registers per thread);
* ``blocks_per_sm`` -- persistent blocks per SM (0 = all that fit); with the
  block size it fixes how many events each thread walks, and the number of
  partial rows the iteration-end kernel reduces;
* ``hist_copies``   -- histogram layout while training: 0 = joint tables of
  dimension pairs, the one layout the sampler has (the per-dimension and
  fixed-point layouts measured slower with the replicated bin table and were
  removed); kept as a field so cached shapes stay comparable.

``tune()`` times every candidate on the integrator's own workload (grid,
integrand, event count) with CUDA events on the launching stream, keeps the
fastest and caches it in a JSON file keyed by (device, algorithm, precision,
n_dim, integrand, event-count bucket, training).  The settings are process-wide
in the native library; an integrator that holds a tuned shape re-applies it
before each of its launches, so integrators with different shapes can be
interleaved.
"""

from __future__ import annotations

import ctypes
import json
import math
import os
import threading

import torch

from . import _native as nat

HIST_CANDIDATES = (0,)
THREAD_CANDIDATES = (1024, 512)
BLOCKS_PER_SM_CANDIDATES = (0, 1)

_lock = threading.Lock()


class LaunchShape:
    """One point of the search space."""

    __slots__ = ("threads", "blocks_per_sm", "hist_copies")

    def __init__(self, threads=1024, blocks_per_sm=0, hist_copies=0):
        if threads not in (512, 1024):
            raise ValueError(f"threads must be 512 or 1024, not {threads}")
        if not 0 <= blocks_per_sm <= 16:
            raise ValueError(f"blocks_per_sm must be in 0..16, not {blocks_per_sm}")
        if hist_copies != 0:
            raise ValueError(f"hist_copies must be 0 (joint pair tables), not {hist_copies}")
        self.threads = int(threads)
        self.blocks_per_sm = int(blocks_per_sm)
        self.hist_copies = int(hist_copies)

    def as_dict(self):
        return {"threads": self.threads, "blocks_per_sm": self.blocks_per_sm, "hist_copies": self.hist_copies}

    @classmethod
    def from_dict(cls, d):
        return cls(int(d["threads"]), int(d["blocks_per_sm"]), int(d["hist_copies"]))

    def __eq__(self, other):
        return isinstance(other, LaunchShape) and self.as_dict() == other.as_dict()

    def __hash__(self):
        return hash((self.threads, self.blocks_per_sm, self.hist_copies))

    def __repr__(self):
        return f"LaunchShape(threads={self.threads}, blocks_per_sm={self.blocks_per_sm}, " \
               f"hist_copies={self.hist_copies})"


DEFAULT_SHAPE = LaunchShape()


_applied = None  # the last shape apply() set (None = unknown)


def apply(shape):
    """Make ``shape`` the native library's current fp32 sampler launch shape."""
    global _applied
    lib = nat.load()
    _applied = None
    nat.check(lib.vf_tune_set(nat.VF_TUNE_F32_THREADS, shape.threads))
    nat.check(lib.vf_tune_set(nat.VF_TUNE_F32_BLOCKS_PER_SM, shape.blocks_per_sm))
    nat.check(lib.vf_tune_set(nat.VF_TUNE_F32_HIST_COPIES, shape.hist_copies))
    _applied = shape


def ensure(shape):
    """``apply(shape)`` unless it is already the shape this module last set."""
    if _applied != shape:
        apply(shape)


def current():
    """The native library's current launch shape."""
    lib = nat.load()
    vals = []
    for key in (nat.VF_TUNE_F32_THREADS, nat.VF_TUNE_F32_BLOCKS_PER_SM, nat.VF_TUNE_F32_HIST_COPIES):
        v = ctypes.c_int(0)
        nat.check(lib.vf_tune_get(key, ctypes.byref(v)))
        vals.append(v.value)
    return LaunchShape(*vals)


def candidates(train=True):
    """Every launch shape to try (a 1024-thread block is alone on its SM, so
    ``blocks_per_sm`` only varies for 512-thread blocks)."""
    hists = HIST_CANDIDATES if train else (0,)
    return [LaunchShape(t, b, h) for h in hists for t in THREAD_CANDIDATES for b in BLOCKS_PER_SM_CANDIDATES
            if not (t == 1024 and b != 0)]


def events_bucket(n_events):
    """Event counts within a factor sqrt(2) share a tuning entry."""
    return int(round(2.0 * math.log2(max(2, int(n_events)))))


def cache_key(device_name, sm_count, alg, precision, n_dim, integrand, n_events, train):
    return "|".join(str(v) for v in (device_name, sm_count, alg, precision, n_dim, integrand,
                                     events_bucket(n_events), int(bool(train))))


def cache_path():
    p = os.environ.get("VEGASFLOW_GB300_TUNE_CACHE")
    if p:
        return p
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "vegasflow_gb300", "launch_shapes.json")


class TuneCache:
    """A JSON file of {key: {"shape": {...}, "ms": t, "default_ms": t0}}."""

    def __init__(self, path=None):
        self.path = path or cache_path()
        self.entries = {}
        try:
            with open(self.path) as fh:
                data = json.load(fh)
            if isinstance(data, dict):
                self.entries = {k: v for k, v in data.items() if isinstance(v, dict) and "shape" in v}
        except (OSError, ValueError):
            self.entries = {}

    def get(self, key):
        e = self.entries.get(key)
        if e is None:
            return None
        try:
            return LaunchShape.from_dict(e["shape"])
        except (KeyError, TypeError, ValueError):
            return None

    def put(self, key, shape, ms, default_ms):
        self.entries[key] = {"shape": shape.as_dict(), "ms": float(ms), "default_ms": float(default_ms)}
        d = os.path.dirname(self.path)
        if d:
            os.makedirs(d, exist_ok=True)
        tmp = f"{self.path}.{os.getpid()}.tmp"
        with open(tmp, "w") as fh:
            json.dump(self.entries, fh, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def _device_id(device):
    props = torch.cuda.get_device_properties(device)
    return props.name, props.multi_processor_count


def rows_for(integrator, shape, train):
    """Partial rows (persistent blocks) the sampler launches under ``shape``."""
    apply(shape)
    rows = ctypes.c_int(0)
    nat.check(nat.load().vf_sample_rows(integrator._ALG, integrator._prec, integrator.n_dim, integrator._int_id,
                                        int(bool(train)), ctypes.byref(rows)))
    return max(1, rows.value)


def time_shape(integrator, shape, train, reps=5, warmup=2):
    """Mean CUDA-event milliseconds of one iteration (sampler launch and
    iteration-end launch) of ``integrator``'s workload under ``shape``.  The
    launches write scratch buffers of their own (partial rows, a copy of the
    grid, history): the integrator's grid, counters and results are untouched."""
    rows = rows_for(integrator, shape, train)
    dev = integrator.device
    k = integrator._n_out
    partials = torch.empty(rows * integrator._width(), dtype=torch.float64, device=dev)
    flags = torch.zeros(1, dtype=torch.int32, device=dev)
    grid = integrator.divisions.detach().clone()
    history = torch.zeros(2 * k, dtype=torch.float64, device=dev)
    avg = torch.zeros(5 * k, dtype=torch.float64, device=dev)
    xmin, xdelta, xdj = integrator._limits_ptrs()
    s = torch.cuda.current_stream(dev)
    call = 0xFFFFFFFF  # a Philox call number no iteration reaches in practice

    def launch():
        nat.call("vf_sample", integrator._ALG, integrator._prec, integrator._grid_ptr(), integrator.n_dim,
                 int(integrator.n_events), 0, float(integrator.xjac), xmin, xdelta, float(xdj), None,
                 integrator._seed, call, int(integrator._int_id), nat.ptr(integrator._params_dev),
                 int(bool(train)), 0, nat.ptr(partials), rows, None, None, None, None, nat.ptr(flags),
                 nat.stream_handle())
        nat.call("vf_iteration_end", nat.ptr(partials), rows, integrator.n_dim, k, int(bool(train)),
                 float(integrator.n_events), 1.5, nat.ptr(grid), None, None, nat.ptr(history), nat.ptr(avg), 0,
                 nat.ptr(flags), nat.stream_handle())

    for _ in range(warmup):
        launch()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(s)
    for _ in range(reps):
        launch()
    end.record(s)
    end.synchronize()
    return start.elapsed_time(end) / reps


def tune(integrator, train=None, cache=None, force=False, reps=5):
    """The fastest launch shape for ``integrator``'s workload (cached).

    Only the fused fp32 VEGAS path (built-in device integrand) has a launch
    shape to choose; for any other configuration this returns ``None``."""
    if not fused_f32(integrator):
        return None
    train = integrator.train if train is None else bool(train)
    name, sms = _device_id(integrator.device)
    key = cache_key(name, sms, integrator._ALG, integrator._prec, integrator.n_dim, integrator._int_id,
                    integrator.n_events, train)
    with _lock:
        cache = cache if cache is not None else TuneCache()
        if not force:
            hit = cache.get(key)
            if hit is not None:
                return hit
        saved = current()
        try:
            times = {}
            for shape in candidates(train):
                times[shape] = time_shape(integrator, shape, train, reps=reps)
            best = min(times, key=times.get)
        finally:
            apply(saved)
        cache.put(key, best, times[best], times.get(DEFAULT_SHAPE, float("nan")))
        return best


def fused_f32(integrator):
    """Whether ``integrator`` launches the fused fp32 VEGAS sampler."""
    return (getattr(integrator, "_FUSED_F32_SAMPLER", False) and integrator.device.type == "cuda"
            and integrator._kind == "device"
            and integrator._prec == nat.VF_PREC_F32 and integrator._ALG == nat.VF_ALG_VEGAS
            and 1 <= getattr(integrator, "_int_id", 0) <= nat.VF_INT_SUM
            and getattr(integrator, "_uniform_source", None) is None)
