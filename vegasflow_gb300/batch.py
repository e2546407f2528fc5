"""Batched VEGAS: many independent integrals per GPU launch.

``VegasBatch`` integrates a list of (n_dim, n_events, device integrand) with
their own grids, all in fp32 fused form: per iteration one persistent sampler
launch over a device work queue of fixed-size event tiles and one batched
iteration-end launch (sums, sigma, weighted average, refinement of every grid
row, counter advance).  The two launches can be captured once in a CUDA graph
and replayed (``graph=True``); every per-iteration quantity (Philox call
counters, history slots, the work queue) lives on the device.

An integral's result depends only on itself (its own Philox stream id, fixed
tile boundaries): the same integral alone and in any mix agrees to the
histogram's float-atomics rounding.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np
import torch

from . import _native as nat
from .configflow import BINS_MAX
from .integrands import CudaIntegrand, DeviceIntegrand
from .utils import capture_guard, preload_kernels

ITEM_DTYPE = np.dtype([("n_events", "<i8"), ("grid_off", "<i8"), ("param_off", "<i8"), ("xjac", "<f8"),
                       ("n_dim", "<i4"), ("integrand", "<i4"), ("stream_id", "<i4"), ("tile0", "<i4"),
                       ("n_tiles", "<i4"), ("train", "<i4"), ("slot", "<i4"), ("pad", "<i4")])
assert ITEM_DTYPE.itemsize == 64

DEFAULT_TILE_EVENTS = 1 << 16


class VegasBatch:
    """Integrate many integrals together.

    ``specs``: iterable of ``(n_dim, n_events, integrand)`` with ``integrand`` a
    built-in ``DeviceIntegrand`` (Gaussian family, Breit-Wigner, prod, sum) or a
    ``CudaIntegrand`` (CUDA source; NVRTC builds a batched sampler around it,
    and its integrals run in a launch of their own, each with its own n_dim and
    the integrand's parameters).
    ``stream_ids``: optional per-integral Philox stream ids (default 0, 1, ...);
    an integral run with the same seed and stream id gives the same numbers in
    any batch."""

    def __init__(self, specs, seed=None, stream_ids=None, train=True, tile_events=DEFAULT_TILE_EVENTS,
                 max_iterations=64, device=None):
        specs = list(specs)
        if not specs:
            raise ValueError("empty batch")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if self.device.type != "cuda":
            raise RuntimeError("VegasBatch runs on a CUDA device only")
        nat.load()
        preload_kernels(self.device)
        self.n_items = len(specs)
        self.seed = int.from_bytes(os.urandom(8), "little") & ((1 << 63) - 1) if seed is None else int(seed)
        self.tile_events = int(tile_events)
        self.hist_cap = int(max_iterations)
        stream_ids = list(range(self.n_items)) if stream_ids is None else list(stream_ids)
        items = np.zeros(self.n_items, dtype=ITEM_DTYPE)
        grids, params = [], []
        tile_item, tile_start, tile_count, tile_row = [], [], [], []
        blk_item, blk_role = [], []
        goff = poff = roff = 0
        self.dims, self.events, self.integrands = [], [], []
        # Launch groups: one sampler launch per (dimension class, program).  The
        # class: integrals with n_dim <= 8 go to the sampler with smaller shared
        # tables and more blocks per SM.  The program: the built-in integrands
        # share one sampler; each CUDA-source integrand has its own.  Items are
        # ordered by group so that each launch's tiles are contiguous; the slot
        # (result index) stays the integral's position in `specs`.
        user = []  # distinct CudaIntegrand objects, in order of appearance
        for i, (n_dim, n_events, integ) in enumerate(specs):
            if isinstance(integ, CudaIntegrand):
                if not any(u is integ for u in user):
                    user.append(integ)
            elif not isinstance(integ, DeviceIntegrand) or not 1 <= integ.integrand_id <= nat.VF_INT_SUM:
                raise TypeError("batched integrals need a built-in DeviceIntegrand or a CudaIntegrand")
            if not 1 <= int(n_dim) <= 16 or int(n_events) < 2:
                raise ValueError(f"integral {i}: n_dim={n_dim}, n_events={n_events}")

        def group_of(i):
            n_dim, _, integ = specs[i]
            prog = next((k + 1 for k, u in enumerate(user) if u is integ), 0)
            return (int(int(n_dim) > 8), prog)

        order = sorted(range(self.n_items), key=group_of)
        group_tiles = {}  # (class, program) -> [first tile, tiles, largest n_dim]
        for pos, i in enumerate(order):  # pos: the integral's place in the items array
            n_dim, n_events, integ = specs[i]
            n_dim, n_events = int(n_dim), int(n_events)
            integ.check_dims(n_dim)
            p = integ.params(n_dim)
            g = group_of(i)
            if g[1]:  # the id of the program's batched sampler for this class
                integ_id = integ.compile_for(nat.VF_ALG_BATCH, nat.VF_PREC_F32, 16 if g[0] else 8)
            else:
                integ_id = integ.integrand_id
            n_tiles = (n_events + self.tile_events - 1) // self.tile_events
            width = 2 + BINS_MAX * n_dim
            gt = group_tiles.setdefault(g, [len(tile_item), 0, 0])
            gt[1] += n_tiles
            gt[2] = max(gt[2], n_dim)
            items[pos] = (n_events, goff, poff, 1.0 / n_events, n_dim, integ_id, stream_ids[i],
                          len(tile_item), n_tiles, int(bool(train)), i, 0)
            for k in range(n_tiles):
                tile_item.append(pos)
                tile_start.append(k * self.tile_events)
                tile_count.append(min(self.tile_events, n_events - k * self.tile_events))
                tile_row.append(roff)
                roff += width
            grids.append(np.linspace(0.0, 1.0, BINS_MAX + 1)[None, :].repeat(n_dim, 0).reshape(-1))
            params.append(p)
            goff += n_dim * (BINS_MAX + 1)
            poff += p.size
            blk_item.extend([pos] * (n_dim + 1))
            blk_role.extend(list(range(n_dim)) + [-1])
        for n_dim, n_events, integ in specs:
            self.dims.append(int(n_dim))
            self.events.append(int(n_events))
            self.integrands.append(integ)
        dev = self.device
        self.max_dim = max(self.dims)
        self.n_tiles = len(tile_item)
        self._items = torch.from_numpy(items.view(np.uint8).copy()).to(dev)
        self.grids = torch.as_tensor(np.concatenate(grids), dtype=torch.float64, device=dev)
        self.params = torch.as_tensor(np.concatenate(params), dtype=torch.float64, device=dev)
        self._grid_off = np.zeros(self.n_items, dtype=np.int64)
        self._grid_off[items["slot"]] = items["grid_off"]  # by slot (the integral's index in specs)
        self._tile_item = torch.as_tensor(tile_item, dtype=torch.int32, device=dev)
        self._tile_start = torch.as_tensor(tile_start, dtype=torch.int64, device=dev)
        self._tile_count = torch.as_tensor(tile_count, dtype=torch.int32, device=dev)
        self._tile_row = torch.as_tensor(tile_row, dtype=torch.int64, device=dev)
        self._blk_item = torch.as_tensor(blk_item, dtype=torch.int32, device=dev)
        self._blk_role = torch.as_tensor(blk_role, dtype=torch.int32, device=dev)
        self.partials = torch.zeros(max(roff, 1), dtype=torch.float64, device=dev)
        self.history = torch.zeros((self.n_items, self.hist_cap, 2), dtype=torch.float64, device=dev)
        self.avg = torch.zeros((self.n_items, 5), dtype=torch.float64, device=dev)
        self._calls = torch.zeros(self.n_items, dtype=torch.int32, device=dev)
        self._iters = torch.zeros(self.n_items, dtype=torch.int32, device=dev)
        self._flags = torch.zeros(1, dtype=torch.int32, device=dev)
        # launches: (first tile, tiles, largest n_dim, JIT id or None); the
        # sampler's persistent grid follows the class's built-in kernel (a JIT
        # build has the same launch bounds and shared memory)
        self._groups = []
        self._blocks = {}
        for (cls, prog), (first, count, md) in sorted(group_tiles.items()):
            jit = int(items[tile_item[first]]["integrand"]) if prog else None
            self._groups.append((first, count, md, jit))
            if md not in self._blocks:
                blocks, smem = ctypes.c_int(0), ctypes.c_int(0)
                nat.check(nat.load().vf_batch_blocks(md, ctypes.byref(blocks), ctypes.byref(smem)))
                self._blocks[md] = blocks.value
        self._queue = torch.zeros(len(self._groups), dtype=torch.int32, device=dev)  # a work counter per launch
        self.blocks = max(self._blocks.values())
        self.iterations_done = 0
        self._graph = None

    # ---------------------------------------------------------------- iterations
    def _launch_iteration(self):
        lib = nat.load()
        s = nat.stream_handle()
        for q, (first, count, md, jit) in enumerate(self._groups):
            args = (nat.ptr(self._items), nat.ptr(self._tile_item[first:]), nat.ptr(self._tile_start[first:]),
                    nat.ptr(self._tile_count[first:]), nat.ptr(self._tile_row[first:]), count, md,
                    nat.ptr(self._queue[q:q + 1]), nat.ptr(self._calls), nat.ptr(self.grids), nat.ptr(self.params),
                    nat.ptr(self.partials), self.seed, nat.ptr(self._flags), self._blocks[md], s)
            if jit is None:
                nat.check(lib.vf_batch_sample(*args))
            else:
                nat.check(lib.vf_batch_sample_jit(jit, *args))
        nat.check(lib.vf_batch_iteration_end(nat.ptr(self._items), nat.ptr(self._blk_item),
                                             nat.ptr(self._blk_role), int(self._blk_item.numel()),
                                             nat.ptr(self._tile_row), nat.ptr(self.partials),
                                             nat.ptr(self.grids), nat.ptr(self.history), nat.ptr(self.avg),
                                             self.hist_cap, nat.ptr(self._iters), nat.ptr(self._calls),
                                             nat.ptr(self._queue), nat.ptr(self._flags), None, s))
        if len(self._groups) > 1:
            self._queue[1:].zero_()  # the iteration end re-arms the first counter

    def reset_average(self):
        """Start a new weighted average (history slots restart at 0); the grids
        and the Philox call counter carry on."""
        self.avg.zero_()
        self._iters.zero_()
        self.iterations_done = 0

    def capture(self):
        """Capture one iteration (2 launches) in a CUDA graph."""
        torch.cuda.synchronize(self.device)
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        # the captured launches must see the counters' device addresses only
        with capture_guard(), torch.cuda.stream(side):
            with torch.cuda.graph(g, stream=side):
                self._launch_iteration()
        torch.cuda.current_stream(self.device).wait_stream(side)
        # capture ran nothing: undo nothing, the counters are untouched
        self._graph = g
        return g

    def run(self, n_iter, graph=False):
        """Run ``n_iter`` iterations of every integral (no host synchronisation)."""
        if self.iterations_done + n_iter > self.hist_cap:
            raise ValueError(f"max_iterations={self.hist_cap} exceeded; call reset_average()")
        if graph and self._graph is None:
            self.capture()
        for _ in range(n_iter):
            if graph:
                self._graph.replay()
            else:
                self._launch_iteration()
        self.iterations_done += n_iter

    def results(self):
        """(mean, sigma, chi2/dof) arrays over the integrals, and the flags word."""
        host = torch.cat([self.avg.reshape(-1), self._flags.to(torch.float64)]).cpu().numpy()
        avg = host[:-1].reshape(self.n_items, 5)
        return avg[:, 2].copy(), avg[:, 3].copy(), avg[:, 4].copy(), int(host[-1])

    def history_host(self):
        """(integrals, iterations, 2) array of every integral's (res, sigma) per iteration."""
        return self.history[:, : self.iterations_done].cpu().numpy()

    def grid(self, i):
        """The current (n_dim, 51) grid of integral ``i`` (a view of the device buffer)."""
        off = int(self._grid_off[i])
        return self.grids[off: off + self.dims[i] * (BINS_MAX + 1)].reshape(self.dims[i], BINS_MAX + 1)

    def total_events(self):
        """Events per iteration over all integrals."""
        return int(sum(self.events))


def c4_specs(n=1024, seed=5):
    """The batched workload: n Gaussians prod_d exp(-(x_d-mu_d)^2/a_d^2) with
    n_dim ~ U{2..16}, events ~ 10^U[4,7], mu_d ~ U[0.3,0.7], a_d ~ U[0.05,0.2]."""
    from .integrands import gauss

    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n):
        d = int(rng.integers(2, 17))
        n_ev = int(10 ** rng.uniform(4, 7))
        mu = rng.uniform(0.3, 0.7, d)
        a = rng.uniform(0.05, 0.2, d)
        specs.append((d, n_ev, gauss(mu, a)))
    return specs
