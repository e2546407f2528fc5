"""Continuous-batching integration server.

Requests (an integrand, n_dim, events per iteration, a target relative sigma
and an iteration cap) arrive over time.  The server keeps every active
request's grid, running average and counters resident on the GPU in a slot
pool and advances *all* active requests by one VEGAS iteration per step -- one
persistent batched sampler launch plus one batched iteration-end launch.
Between steps it retires the requests that reached their target (or their
iteration cap) and admits waiting ones while slots and the HBM budget allow,
so requests that arrive while others are on the GPU join at the next step
and their work overlaps with everyone else's.

An integral's numbers depend only on itself (its Philox stream id and fixed
event tiles): a request gives the same result alone and in any mix, up to the
rounding of the histogram's float atomics.

Integrands are the built-in device integrands, which share one sampler, or
CUDA-source integrands (``integrands.cuda_integrand``), compiled by NVRTC when
the request is submitted into a batched sampler of their own: each step then
launches one sampler per (program, dimension class) present.

Failures stay with the request they concern, never the server: a request that
cannot be served (unsupported integrand or dimension, CUDA source that does not
compile, larger than the whole HBM budget) is rejected at submission; a request can be cancelled, or expire
after its ``timeout``, at the next step boundary; a device allocation that
fails (growing the partial-row buffer, admitting requests) fails the requests
it was for and the server carries on with the others.  ``fault_hook``
(host-side fault injection for tests) is called at those points and may raise.
Every finished request carries a ``status`` (converged, finished, cancelled,
expired, rejected, failed) and, for the last three, an ``error``.
"""

from __future__ import annotations

import ctypes
import itertools
import math
import os
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as nat
from .utils import preload_kernels
from .batch import DEFAULT_TILE_EVENTS, ITEM_DTYPE
from .configflow import BINS_MAX
from .integrands import CudaIntegrand, DeviceIntegrand

MAX_DIM = 16
PARAMS_PER_SLOT = 2 * MAX_DIM + 2


@dataclass
class Request:
    """One integration request: integrand, n_dim, events per iteration, the target
    relative sigma and iteration cap, its arrival time (seconds) and optional timeout;
    the server fills in the result, status and timings."""

    n_dim: int
    n_events: int
    integrand: DeviceIntegrand
    target_rel_sigma: float = 1e-3
    max_iterations: int = 20
    arrival: float = 0.0
    rid: int = -1
    # filled in by the server
    result: float = float("nan")
    sigma: float = float("nan")
    iterations: int = 0
    converged: bool = False
    admitted: float = float("nan")
    finished: float = float("nan")
    slot: int = -1
    timeout: float = float("inf")  # seconds after arrival
    status: str = "new"           # waiting, active, then a final status (see the module docstring)
    error: str = ""
    exact: float = field(default=float("nan"), repr=False)
    program: int = field(default=0, repr=False)  # 0: the built-in sampler; else its batched JIT sampler's id

    @property
    def latency(self):
        return self.finished - self.arrival


# Tile sizes of served requests: a persistent sampler block processes one tile
# (256 threads), so a request cut into few large tiles runs on few SMs and its
# iteration takes as long as one block needs for a whole tile (~250 us for 64K
# events).  A served request is cut into about SERVE_TILES tiles of between
# SERVE_TILE_MIN and DEFAULT_TILE_EVENTS events (a multiple of 256): small
# requests spread over the GPU, large ones keep tiles big enough that the
# per-tile work (histogram clear and flush, the partial row) stays small.  The
# size depends only on the request's own event count, so its result does not
# depend on the other requests.
SERVE_TILES = 512
SERVE_TILE_MIN = 2048


def serving_tile_events(n_events):
    """Events per tile of a served request of ``n_events`` events (scalar or array)."""
    n = np.asarray(n_events, dtype=np.int64)
    t = (n + SERVE_TILES - 1) // SERVE_TILES
    t = (t + 255) // 256 * 256
    return np.minimum(DEFAULT_TILE_EVENTS, np.maximum(SERVE_TILE_MIN, t))


def step_tables(n_events, n_dim, slots, stream_ids, integrand_ids, grid_off, param_off, tile_events, train=True):
    """The per-step device tables for the active requests (host side, vectorised):
    items, tiles (item, first event, count, partial-row offset) and the
    iteration-end block table (item, role).  ``tile_events``: one tile size for
    every request, or one per request."""
    n_events = np.asarray(n_events, dtype=np.int64)
    n_dim = np.asarray(n_dim, dtype=np.int64)
    n = n_events.size
    tile_events = np.broadcast_to(np.asarray(tile_events, dtype=np.int64), n_events.shape)
    n_tiles = (n_events + tile_events - 1) // tile_events
    tile0 = np.concatenate([[0], np.cumsum(n_tiles)[:-1]])[:n].astype(np.int64)
    total = int(n_tiles.sum())
    tile_item = np.repeat(np.arange(n, dtype=np.int32), n_tiles)
    k = np.arange(total, dtype=np.int64) - np.repeat(tile0, n_tiles)
    tile_size = np.repeat(tile_events, n_tiles)
    tile_start = k * tile_size
    tile_count = np.minimum(tile_size, np.repeat(n_events, n_tiles) - tile_start).astype(np.int32)
    width = 2 + BINS_MAX * np.repeat(n_dim, n_tiles)
    tile_row = np.concatenate([[0], np.cumsum(width)[:-1]])[:total].astype(np.int64)
    rows_total = int(width.sum())
    items = np.zeros(n, dtype=ITEM_DTYPE)
    items["n_events"] = n_events
    items["grid_off"] = grid_off
    items["param_off"] = param_off
    items["xjac"] = 1.0 / n_events
    items["n_dim"] = n_dim
    items["integrand"] = integrand_ids
    items["stream_id"] = stream_ids
    items["tile0"] = tile0
    items["n_tiles"] = n_tiles
    items["train"] = int(bool(train))
    items["slot"] = slots
    blk_item = np.repeat(np.arange(n, dtype=np.int32), n_dim + 1)
    starts = np.concatenate([[0], np.cumsum(n_dim + 1)[:-1]])[:n]
    blk_role = (np.arange(int((n_dim + 1).sum())) - np.repeat(starts, n_dim + 1)).astype(np.int32)
    last = starts + n_dim
    blk_role[last] = -1
    return dict(items=items, tile_item=tile_item, tile_start=tile_start, tile_count=tile_count,
                tile_row=tile_row, blk_item=blk_item, blk_role=blk_role, rows_total=rows_total,
                n_tiles=total)


def launch_groups(act, n_tiles, small_blocks):
    """The sampler launches of a step over the active requests ``act`` (ordered
    by (program, n_dim > 8); ``n_tiles`` their tile counts): a list of (first
    tile, tiles, max_dim, JIT id or None), one per run of equal (program,
    dimension class).  When the built-in sampler has both classes and one of
    them has fewer tiles than ``small_blocks`` (the general sampler's persistent
    grid), they share one launch of the general sampler."""
    groups = []
    first = 0
    for (prog, high), run in itertools.groupby(range(len(act)), key=lambda k: (act[k].program, act[k].n_dim > 8)):
        count = int(sum(int(n_tiles[k]) for k in run))
        groups.append((first, count, MAX_DIM if high else 8, prog or None))
        first += count
    if (len(groups) >= 2 and groups[0][3] is None and groups[1][3] is None and groups[0][2] == 8
            and min(groups[0][1], groups[1][1]) < small_blocks):
        groups[0:2] = [(0, groups[0][1] + groups[1][1], MAX_DIM, None)]
    return groups


def request_footprint(n_dim, n_events, tile_events=None, hist_cap=32):
    """Device bytes a request holds while active: its slot (grid, parameters,
    history, average, counters) and its partial rows (``tile_events`` None: the
    served tile size of ``serving_tile_events``)."""
    if tile_events is None:
        tile_events = int(serving_tile_events(n_events))
    n_tiles = (n_events + tile_events - 1) // tile_events
    rows = n_tiles * (2 + BINS_MAX * n_dim) * 8
    slot = (MAX_DIM * (BINS_MAX + 1) + PARAMS_PER_SLOT + 2 * hist_cap + 5) * 8 + 8
    return rows + slot + n_tiles * 24


def percentile(values, q):
    """The ``q``-th percentile of ``values`` (NaN for an empty list)."""
    v = np.sort(np.asarray(values, dtype=np.float64))
    if v.size == 0:
        return float("nan")
    return float(np.percentile(v, q))


class VegasServer:
    """Continuous batching over a GPU slot pool.

    ``max_slots`` bounds the number of concurrently active requests;
    ``hbm_budget`` (bytes) bounds the device memory they hold (admission
    control); ``seed`` keys every request's Philox stream (with its request id as
    stream id)."""

    def __init__(self, max_slots=2048, hbm_budget=150e9, tile_events=None, seed=1234,
                 hist_cap=32, device=None, fault_hook=None):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if self.device.type != "cuda":
            raise RuntimeError("VegasServer runs on a CUDA device only")
        nat.load()
        preload_kernels(self.device)
        self.max_slots = int(max_slots)
        self.hbm_budget = float(hbm_budget)
        self.tile_events = None if tile_events is None else int(tile_events)  # None: per request
        self.seed = int(seed)
        self.hist_cap = int(hist_cap)
        dev = self.device
        self.grids = torch.zeros(self.max_slots * MAX_DIM * (BINS_MAX + 1), dtype=torch.float64, device=dev)
        self.params = torch.zeros(self.max_slots * PARAMS_PER_SLOT, dtype=torch.float64, device=dev)
        self.history = torch.zeros((self.max_slots, self.hist_cap, 2), dtype=torch.float64, device=dev)
        self.avg = torch.zeros((self.max_slots, 5), dtype=torch.float64, device=dev)
        self.iters = torch.zeros(self.max_slots, dtype=torch.int32, device=dev)
        self.calls = torch.zeros(self.max_slots, dtype=torch.int32, device=dev)
        self._queue = torch.zeros(4, dtype=torch.int32, device=dev)  # a work counter per sampler launch (grows)
        self._flags = torch.zeros(1, dtype=torch.int32, device=dev)
        self.partials = torch.zeros(1 << 20, dtype=torch.float64, device=dev)
        self._blocks = {}
        for md in (8, MAX_DIM):  # the samplers of the two dimension classes
            blocks, smem = ctypes.c_int(0), ctypes.c_int(0)
            nat.check(nat.load().vf_batch_blocks(md, ctypes.byref(blocks), ctypes.byref(smem)))
            self._blocks[md] = blocks.value
        self.blocks = self._blocks[MAX_DIM]
        self._uniform_row = torch.as_tensor(np.linspace(0.0, 1.0, BINS_MAX + 1), dtype=torch.float64, device=dev)
        # the active set's device tables and launch arguments (rebuilt when it changes),
        # their pinned staging buffer, and pinned mirrors for the per-step state read
        self._prep = None
        self._tab_host = torch.empty(0, dtype=torch.uint8)
        self._tab_dev = torch.empty(0, dtype=torch.uint8, device=dev)
        # per step, the iteration end writes each active request's (mean, sigma,
        # iterations) here, in pinned host memory the device addresses directly
        self._status = torch.zeros((self.max_slots, 3), dtype=torch.float64).pin_memory()
        self.free_slots = list(range(self.max_slots - 1, -1, -1))
        self.active = []          # requests on the GPU
        self.waiting = []         # arrived, not admitted yet
        self.done = []
        self.bytes_in_use = 0.0
        self.events_done = 0
        self.steps = 0
        self._next_rid = 0
        self._cancel = set()
        self.fault_hook = fault_hook

    # ---------------------------------------------------------------- admission
    def _fault(self, event, **info):
        if self.fault_hook is not None:
            self.fault_hook(event, **info)

    def _finish(self, req, status, now, error=""):
        """Retire ``req`` with a final status (freeing its slot if it held one)."""
        if req.slot >= 0:
            self.free_slots.append(req.slot)
            self.bytes_in_use -= req._footprint
            req.slot = -1
        req.status = status
        req.error = error
        req.converged = status == "converged"
        req.finished = now
        self.done.append(req)

    def submit(self, req: Request, now=None):
        """Queue ``req``; a request that can never be served is rejected here
        (status ``rejected``) instead of raising."""
        if req.rid < 0:
            req.rid = self._next_rid
        self._next_rid = max(self._next_rid, req.rid + 1)
        now = req.arrival if now is None else now
        reason = ""
        integ = req.integrand
        user = isinstance(integ, CudaIntegrand)
        if not user and (not isinstance(integ, DeviceIntegrand)
                         or not nat.VF_INT_SYMGAUSS <= integ.integrand_id <= nat.VF_INT_SUM):
            reason = "batched serving takes built-in device integrands or CUDA-source integrands"
        elif not 1 <= req.n_dim <= MAX_DIM:
            reason = f"n_dim={req.n_dim} outside 1..{MAX_DIM}"
        elif req.n_events < 2:
            reason = f"n_events={req.n_events} < 2"
        elif request_footprint(req.n_dim, req.n_events, self.tile_events, self.hist_cap) > self.hbm_budget:
            reason = "larger than the HBM budget"
        elif user and integ.params(req.n_dim).size > PARAMS_PER_SLOT:
            reason = f"more than {PARAMS_PER_SLOT} integrand parameters"
        else:
            try:
                integ.check_dims(req.n_dim)
                if user:  # the program's batched sampler for the request's dimension class
                    req.program = integ.compile_for(nat.VF_ALG_BATCH, nat.VF_PREC_F32, MAX_DIM if req.n_dim > 8 else 8)
            except ValueError as exc:
                reason = str(exc)
            except nat.VegasGB300Error as exc:
                reason = f"the CUDA integrand did not compile: {exc}"
        if reason:
            self._finish(req, "rejected", now, reason)
            return False
        req.status = "waiting"
        self.waiting.append(req)
        return True

    def cancel(self, rid):
        """Cancel request ``rid``: a waiting one at once, an active one at the
        next step boundary (its result so far is kept)."""
        self._cancel.add(int(rid))

    def _triage(self, now):
        """Cancellations and expiries, between steps (no expiry without a clock)."""

        def expired(req):
            return math.isfinite(now) and now >= req.arrival + req.timeout

        keep = []
        for req in self.waiting:
            if req.rid in self._cancel:
                self._finish(req, "cancelled", now, "cancelled before admission")
            elif expired(req):
                self._finish(req, "expired", now, "timed out before admission")
            else:
                keep.append(req)
        self.waiting = keep
        keep = []
        for req in self.active:
            if req.rid in self._cancel:
                self._finish(req, "cancelled", now, "cancelled")
            elif expired(req):
                self._finish(req, "expired", now, f"timed out after {req.iterations} iterations")
            else:
                keep.append(req)
        self.active = keep

    def _admit(self, now):
        admitted = []
        keep = []
        for req in self.waiting:
            fp = request_footprint(req.n_dim, req.n_events, self.tile_events, self.hist_cap)
            if self.free_slots and self.bytes_in_use + fp <= self.hbm_budget:
                req.slot = self.free_slots.pop()
                req.admitted = now
                req._footprint = fp
                self.bytes_in_use += fp
                admitted.append(req)
            else:
                keep.append(req)
        self.waiting = keep
        if not admitted:
            return
        try:
            self._fault("admit", requests=admitted)
            self._load_slots(admitted)
        except (RuntimeError, MemoryError) as exc:  # a device allocation failed: fail these requests only
            for req in admitted:
                self._finish(req, "failed", now, f"admission failed: {exc}")
            return
        for req in admitted:
            req.status = "active"
        self.active.extend(admitted)

    def _load_slots(self, admitted):
        """Initialise the slots of newly admitted requests (uniform grid,
        parameters, cleared history, average and counters)."""
        slots = torch.as_tensor([r.slot for r in admitted], dtype=torch.int64, device=self.device)
        grid_rows = self.grids.view(self.max_slots, MAX_DIM, BINS_MAX + 1)
        grid_rows[slots] = self._uniform_row
        p = np.zeros((len(admitted), PARAMS_PER_SLOT))
        for i, r in enumerate(admitted):
            pr = r.integrand.params(r.n_dim)
            p[i, : pr.size] = pr
        self.params.view(self.max_slots, PARAMS_PER_SLOT)[slots] = torch.as_tensor(p, device=self.device)
        self.history[slots] = 0.0
        self.avg[slots] = 0.0
        self.iters[slots] = 0
        self.calls[slots] = 0

    # ---------------------------------------------------------------- one step
    def _tables(self, act):
        return step_tables([r.n_events for r in act], [r.n_dim for r in act], [r.slot for r in act],
                           [r.rid for r in act], [r.program or r.integrand.integrand_id for r in act],
                           [r.slot * MAX_DIM * (BINS_MAX + 1) for r in act],
                           [r.slot * PARAMS_PER_SLOT for r in act],
                           self.tile_events if self.tile_events is not None
                           else serving_tile_events([r.n_events for r in act]))

    _TABLES = ("items", "tile_item", "tile_start", "tile_count", "tile_row", "blk_item", "blk_role")

    def _prepare(self, act, t, stream):
        """Device tables and launch arguments of the active set ``act`` (tables
        ``t``): the seven tables packed into one pinned staging buffer and sent
        with one copy, and every launch's ctypes arguments built once.  Each step
        ends with a stream synchronize, so the staging and table buffers are idle
        whenever they are rewritten."""
        blobs = [t["items"].view(np.uint8)] + [np.ascontiguousarray(t[k]).view(np.uint8) for k in self._TABLES[1:]]
        offs, total = [], 0
        for b in blobs:
            offs.append(total)
            total += (b.size + 15) // 16 * 16
        if self._tab_host.numel() < total:
            cap = max(total, 2 * self._tab_host.numel(), 1 << 16)
            self._tab_host = torch.empty(cap, dtype=torch.uint8).pin_memory()
            self._tab_dev = torch.empty(cap, dtype=torch.uint8, device=self.device)
        h = self._tab_host.numpy()
        for b, o in zip(blobs, offs):
            h[o:o + b.size] = b.reshape(-1)
        self._tab_dev[:total].copy_(self._tab_host[:total], non_blocking=True)
        base = self._tab_dev.data_ptr()
        at = {k: base + o for k, o in zip(self._TABLES, offs)}
        vp = ctypes.c_void_p
        lib = nat.load()
        groups = launch_groups(act, t["items"]["n_tiles"], self._blocks[MAX_DIM])
        if len(groups) > self._queue.numel():
            self._queue = torch.zeros(2 * len(groups), dtype=torch.int32, device=self.device)
        launches = []
        for q, (first, count, md, jit) in enumerate(groups):
            args = (vp(at["items"]), vp(at["tile_item"] + 4 * first), vp(at["tile_start"] + 8 * first),
                    vp(at["tile_count"] + 4 * first), vp(at["tile_row"] + 8 * first), count, md,
                    vp(self._queue.data_ptr() + 4 * q), nat.ptr(self.calls), nat.ptr(self.grids),
                    nat.ptr(self.params), nat.ptr(self.partials), self.seed, nat.ptr(self._flags),
                    self._blocks[md], stream)
            launches.append((lib.vf_batch_sample, args) if jit is None else
                            (lib.vf_batch_sample_jit, (jit,) + args))
        launches.append((lib.vf_batch_iteration_end,
                         (vp(at["items"]), vp(at["blk_item"]), vp(at["blk_role"]), int(t["blk_item"].size),
                          vp(at["tile_row"]), nat.ptr(self.partials), nat.ptr(self.grids), nat.ptr(self.history),
                          nat.ptr(self.avg), self.hist_cap, nat.ptr(self.iters), nat.ptr(self.calls),
                          nat.ptr(self._queue), nat.ptr(self._flags), vp(self._status.data_ptr()), stream)))
        return {"key": self._prep_key(act, stream), "launches": launches, "n_groups": len(groups),
                "events": int(sum(r.n_events for r in act))}

    def _prep_key(self, act, stream):
        """Everything the step's tables and launch arguments are built from: per
        request (in launch order) its stream id, slot, event and dimension counts
        and program, and the buffers the arguments point into."""
        reqs = tuple((r.rid, r.slot, r.n_events, r.n_dim, r.program or r.integrand.integrand_id) for r in act)
        return (reqs, stream.value, self.partials.data_ptr(), self._queue.data_ptr())

    def step(self, now_fn):
        """Advance every active request by one iteration, then retire finished ones."""
        # ordered by (program, dimension class): each run of tiles goes to one
        # sampler launch (n_dim <= 8: the class with smaller shared tables)
        act = sorted(self.active, key=lambda r: (r.program, r.n_dim > 8))
        stream = nat.stream_handle()
        prep = self._prep
        if prep is None or prep["key"] != self._prep_key(act, stream):
            t = self._tables(act)
            if t["rows_total"] > self.partials.numel():
                try:
                    self._fault("grow", rows=t["rows_total"])
                    self.partials = torch.zeros(int(t["rows_total"] * 1.5), dtype=torch.float64, device=self.device)
                except (RuntimeError, MemoryError) as exc:
                    # no room for this step's partial rows: fail the newest requests until the
                    # rest fit the buffer there is, and take the step with those
                    now = now_fn()
                    while act and t["rows_total"] > self.partials.numel():
                        self._finish(act.pop(), "failed", now, f"device allocation failed: {exc}")
                        t = self._tables(act)
                    self.active = act
                    if not act:
                        return
            prep = self._prep = self._prepare(act, t, stream)
        for fn, args in prep["launches"]:
            nat.check(fn(*args))
        if prep["n_groups"] > 1:
            self._queue[1:prep["n_groups"]].zero_()  # the other launches' counters (the iteration end re-arms the first)
        # the iteration end has written every active request's state into pinned
        # host memory: one synchronize, no copy
        torch.cuda.current_stream(self.device).synchronize()
        now = now_fn()
        n = len(act)
        st = self._status.numpy()[:n]
        means, sigmas, its = st[:, 0], st[:, 1], st[:, 2].astype(np.int64)
        target = np.array([r.target_rel_sigma for r in act]) if n > 1 else act[0].target_rel_sigma
        cap = np.array([r.max_iterations for r in act]) if n > 1 else act[0].max_iterations
        with np.errstate(invalid="ignore", divide="ignore"):
            conv = np.isfinite(means) & np.isfinite(sigmas) & (means != 0.0) & (sigmas / np.abs(means) <= target)
        done = conv | (its >= cap)
        self.events_done += prep["events"]
        self.steps += 1
        for r, m, sg, it in zip(act, means.tolist(), sigmas.tolist(), its.tolist()):
            r.iterations, r.result, r.sigma = it, m, sg
        if done.any():
            still = []
            for r, c, d in zip(act, conv.tolist(), done.tolist()):
                if d:
                    self._finish(r, "converged" if c else "finished", now)
                else:
                    still.append(r)
            self.active = still
        else:
            self.active = act

    # ---------------------------------------------------------------- the loop
    def run(self, requests, realtime=True, time_limit=None):
        """Serve ``requests`` (sorted by arrival).  With ``realtime`` the arrival
        times are wall-clock offsets from the start; requests are admitted when
        they have arrived.  Returns the metrics dict."""
        pending = sorted(requests, key=lambda r: r.arrival)
        for i, r in enumerate(pending):
            if r.rid < 0:
                r.rid = i
        t0 = time.perf_counter()
        now_fn = (lambda: time.perf_counter() - t0) if realtime else (lambda: float("inf"))
        pi = 0
        busy = 0.0
        while pi < len(pending) or self.waiting or self.active:
            now = now_fn()
            while pi < len(pending) and pending[pi].arrival <= now:
                self.submit(pending[pi], now=now)
                pi += 1
            self._triage(now)
            if self.waiting:
                self._admit(now)
            if not self.active:
                if pi < len(pending):
                    wait = pending[pi].arrival - now_fn()
                    if wait > 0:
                        time.sleep(min(wait, 0.01))
                    continue
                if self.waiting:  # every waiting request fits an empty pool: admission retries
                    continue
                break
            ts = time.perf_counter()
            self.step(now_fn)
            busy += time.perf_counter() - ts
            if time_limit is not None and now_fn() > time_limit:
                break
        wall = time.perf_counter() - t0
        if not realtime:
            for r in self.done:
                r.finished = r.arrival  # no clock: latencies are not measured
        served = [r for r in self.done if r.status in ("converged", "finished")]
        lat = [r.latency for r in served]
        lat_conv = [r.latency for r in served if r.converged]
        flags = int(self._flags.item())
        by_status = {}
        for r in self.done:
            by_status[r.status] = by_status.get(r.status, 0) + 1
        return {"requests": len(self.done), "converged": int(sum(r.converged for r in self.done)),
                "status": by_status,
                "p50_latency_s": percentile(lat, 50), "p99_latency_s": percentile(lat, 99),
                "mean_latency_s": float(np.mean(lat)) if lat else float("nan"),
                # requests that reached their target sigma (the rest stopped at the iteration cap)
                "p50_converged_s": percentile(lat_conv, 50), "p99_converged_s": percentile(lat_conv, 99),
                "reached_target_fraction": len(lat_conv) / len(served) if served else float("nan"),
                "events": self.events_done, "wall_s": wall, "busy_s": busy,
                "events_per_s": self.events_done / wall if wall > 0 else float("nan"),
                "steps": self.steps, "flags": flags}


def poisson_workload(rate=200.0, duration=60.0, seed=9, bw_fraction=0.2, target_rel_sigma=1e-3,
                     max_iterations=20):
    """Synthetic request stream: Poisson arrivals at ``rate``/s over ``duration``
    seconds; each request a per-dimension Gaussian (n_dim ~ U{2..16}, events ~
    10^U[4,7], mu ~ U[0.3,0.7], a ~ U[0.05,0.2]), a fraction replaced by the 6-D
    Breit-Wigner x linear integrand (c_d from seed 3, 2e6 events)."""
    from .integrands import breit_wigner, gauss

    rng = np.random.default_rng(seed)
    c = np.random.default_rng(3).random(5)
    t = 0.0
    reqs = []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        if rng.random() < bw_fraction:
            reqs.append(Request(6, 2_000_000, breit_wigner(c), target_rel_sigma, max_iterations, t))
        else:
            d = int(rng.integers(2, 17))
            n = int(10 ** rng.uniform(4, 7))
            reqs.append(Request(d, n, gauss(rng.uniform(0.3, 0.7, d), rng.uniform(0.05, 0.2, d)),
                                target_rel_sigma, max_iterations, t))
    for i, r in enumerate(reqs):
        r.rid = i
    return reqs
