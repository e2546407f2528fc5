"""The Monte Carlo driver: ``MonteCarloFlow`` (vegasflow monte_carlo.py:95-741).

Same public surface as the reference: ``MonteCarloFlow(n_dim, n_events,
events_limit, list_devices, verbose, xmin, xmax)``, ``compile(integrand,
compilable, signature, trace, check)``, ``run_integration(n_iter, log_time,
histograms)``, ``run_event``, ``generate_random_array``, ``set_seed``, the
``n_events`` / ``events_per_run`` / ``history`` / ``xjac`` properties, and the
``wrapper`` / ``sampler`` helpers, ``make_differentiable`` and the device-pool
methods (``get_device`` / ``release_device`` / ``device_run`` over the one GPU).
Extra keyword arguments: ``precision`` ("fp64" = the reference's float64
arithmetic, "fp32" = the fused fp32 form), ``device``, ``seed``, ``autotune``
(time the fp32 sampler's launch shapes on the workload and cache the winner) and
``cuda_graph`` (iterations of device integrands as replays of one captured CUDA
graph).

Execution model (one GPU):
  * an integrand built with ``vegasflow_gb300.integrands`` runs *inside* the
    sampler kernel: one launch per iteration samples, maps, evaluates and
    reduces every event (``events_limit`` needs no chunking: the kernel keeps no
    per-event state in memory);
  * a torch callable runs on the sampler's x in HBM, chunk by chunk
    (``events_per_run`` events per chunk, as the reference), followed by a
    reduction kernel;
  * per iteration one iteration-end kernel sums the block partials, computes
    sigma, the running weighted average and chi^2, and refines the grid.  No
    host synchronisation happens until ``run_integration`` returns (or each
    iteration when ``verbose`` prints it).
"""

from __future__ import annotations

import copy
import inspect
import logging
import os
import threading
import time
from abc import ABC, abstractmethod

import numpy as np
import torch

from . import _native as nat
from . import autotune
from .configflow import (
    ALPHA,
    BINS_MAX,
    DEFAULT_ACTIVE_DEVICES,
    DEFAULT_PRECISION,
    DTYPE,
    MAX_EVENTS_LIMIT,
)
from .integrands import DeviceIntegrand

logger = logging.getLogger("vegasflow.monte_carlo")

# Iterations captured in one CUDA graph at most (cuda_graph=True, run_integration
# without per-iteration logging): one graph launch and one host call per
# GRAPH_UNROLL iterations.  Measured on the 4-D Gaussian at 1e6 events: a replay
# of one iteration costs ~6 us of host time and the graph launches add gaps.
GRAPH_UNROLL = 8


class _nvtx:
    """An NVTX range (for Nsight timelines) around a block of host calls when
    VEGASFLOW_NVTX=1; nothing otherwise."""

    def __init__(self, name):
        self.name = name
        self.on = os.environ.get("VEGASFLOW_NVTX", "0") == "1"

    def __enter__(self):
        if self.on:
            torch.cuda.nvtx.range_push(self.name)

    def __exit__(self, *exc):
        if self.on:
            torch.cuda.nvtx.range_pop()

VF_MAX_DIM = 16


def print_iteration(it, res, error, extra="", threshold=0.1):
    """monte_carlo.py:61-69."""
    if res < threshold:
        return f"Result for iteration {it}: {res:.3e} +/- {error:.3e}" + extra
    return f"Result for iteration {it}: {res:.4f} +/- {error:.4f}" + extra


# events per launched sampler block: at least EVENTS_PER_BLOCK_MIN while the
# blocks do not cover the SMs, then EVENTS_PER_BLOCK_TARGET (measured at 1e6
# events: fewer, fuller blocks were 5-10% faster -- every block stages its table,
# clears and reads back its histogram and adds a partial row to reduce)
EVENTS_PER_BLOCK_MIN = 1024
EVENTS_PER_BLOCK_TARGET = 4096


def _chunk_sizes(n_events, events_per_run):
    """monte_carlo.py:437-452."""
    out = []
    left = int(n_events)
    while left > 0:
        out.append(min(left, events_per_run))
        left -= events_per_run
    return out


def _random_seed():
    return int.from_bytes(os.urandom(8), "little") & ((1 << 63) - 1)


class MonteCarloFlow(ABC):
    """Parent class of the integrators (monte_carlo.py:95)."""

    _CAN_RUN_VECTORIAL = False
    _ALG = nat.VF_ALG_PLAIN
    _FUSED_F32_SAMPLER = False  # launches the fused fp32 VEGAS sampler (has a launch shape)
    _GRAPH_ITERATIONS = False  # one iteration is vf_iteration_dev (CUDA-graph replayable)

    def __init__(self, n_dim, n_events, events_limit=MAX_EVENTS_LIMIT,
                 list_devices=DEFAULT_ACTIVE_DEVICES, verbose=True, xmin=None, xmax=None,
                 precision=None, device=None, seed=None, autotune=False, cuda_graph=False, **kwargs):
        if "simplify_signature" in kwargs:
            logger.warning("simplify_signature is deprecated and will be removed")
        self.n_dim = int(n_dim)
        if not 1 <= self.n_dim <= VF_MAX_DIM:
            raise ValueError(f"n_dim={n_dim}: the GB300 sampler supports 1 to {VF_MAX_DIM} dimensions")
        self._integrand = None
        self._tf_integrand = None
        self.event = None
        self._verbose = verbose
        self._history = []
        self._n_events = int(n_events)
        self._events_limit = int(events_limit)
        self._events_per_run = min(self._events_limit, self._n_events)
        self._compilation_arguments = None
        self._vectorial = False
        self._n_out = 1
        self.distribute = False
        self._pass_weight = False
        self.list_devices = list_devices
        self.devices = None  # the device pool (get_device / release_device): this integrator's GPU
        self.lock = threading.Lock()
        self.precision = (precision or DEFAULT_PRECISION).lower()
        if self.precision not in ("fp64", "fp32"):
            raise ValueError(f"precision must be 'fp64' or 'fp32', not {precision!r}")
        self._prec = nat.VF_PREC_F64 if self.precision == "fp64" else nat.VF_PREC_F32
        self._rdtype = torch.float64 if self.precision == "fp64" else torch.float32
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() \
                else torch.device("cpu")
        self.device = torch.device(device)
        self._seed = _random_seed() if seed is None else int(seed)
        self._call_ctr = 0
        self._uniform_source = None
        self._kind = None
        self._rows = 0
        self._ws = {}
        self._it = 0
        self._autotune = bool(autotune)
        self._shape = None
        self._cuda_graph = bool(cuda_graph)
        self._differentiable = False
        self._graph = None
        self._graph_key = None
        self._graphs_unrolled = {}

        if xmin is not None or xmax is not None:  # monte_carlo.py:159-175
            if xmin is None or xmax is None:
                raise ValueError(
                    "Both xmin and xmax must be provided if the integration limits are to change")
            if not (len(xmin) == len(xmax) == n_dim):
                raise ValueError("The integration limits must be given for all dimensions")
            self._xmin_np = np.asarray(xmin, dtype=np.float64)
            self._xdelta_np = np.asarray(xmax, dtype=np.float64) - self._xmin_np
            if any(self._xdelta_np < 0.0):
                raise ValueError(f"No xmin ({xmin}) can be bigger than xmax ({xmax})")
            jac = self._xdelta_np[0]
            for d in range(1, self.n_dim):
                jac = jac * self._xdelta_np[d]
            self._xdeltajac = float(jac)
            self._xmin = torch.as_tensor(self._xmin_np, device=self.device)
            self._xdelta = torch.as_tensor(self._xdelta_np, device=self.device)
        else:
            self._xmin = self._xdelta = None
            self._xmin_np = self._xdelta_np = None
            self._xdeltajac = None

    # ---------------------------------------------------------------- properties
    @property
    def n_events(self):
        """Number of events to run in a single iteration."""
        return self._n_events

    @n_events.setter
    def n_events(self, val):
        self._n_events = int(val)
        self.events_per_run = self._events_limit
        self._recompile()

    @property
    def events_per_run(self):
        """Events per step of a torch-callable integrand (memory knob)."""
        return self._events_per_run

    @events_per_run.setter
    def events_per_run(self, val):
        self._events_per_run = min(int(val), self.n_events)
        if self._events_per_run and self.n_events % self._events_per_run != 0:
            logger.warning(
                f"The number of events per run step {self._events_per_run} doesn't perfectly"
                f"divide the number of events {self.n_events}, which can harm performance")

    @property
    def history(self):
        """List of (result, error, histograms) per iteration."""
        return self._history

    @property
    def xjac(self):
        """The default Jacobian is 1 / total number of events."""
        return 1.0 / self.n_events

    # ---------------------------------------------------------------- seeds / rng
    def set_seed(self, seed):
        """Seed the Philox stream (key = seed; the per-iteration counter restarts)."""
        self._seed = int(seed)
        self._call_ctr = 0

    def _next_call(self):
        c = self._call_ctr
        self._call_ctr += 1
        return c & 0xFFFFFFFF

    def set_uniform_source(self, source):
        """Inject uniforms: ``source(n, n_dim)`` returns an (n, n_dim) float64 device
        tensor of post-affine uniforms (U[TECH_CUT, 1-TECH_CUT)) used instead of the
        in-kernel Philox stream for the next chunks; ``None`` restores Philox."""
        self._uniform_source = source

    # ---------------------------------------------------------------- abstract hooks
    @abstractmethod
    def _run_iteration(self):
        """Run one iteration (``self.n_events``) of the integration."""

    @abstractmethod
    def _run_event(self, integrand, ncalls=None):
        """Run one chunk of events; returns the accumulables."""

    def _digest_random_generation(self, xrand, *args):
        return xrand, 1.0

    def _can_run_vectorial(self, expected_shape=None):
        return self._CAN_RUN_VECTORIAL

    def _grid_ptr(self):
        return None

    def _train_now(self):
        return False

    # ---------------------------------------------------------------- device helpers
    def _require_gpu(self):
        if self.device.type != "cuda":
            raise RuntimeError("vegasflow_gb300 runs on a CUDA device only (no CPU fallback); "
                               f"this integrator was created on {self.device}")
        nat.load()

    def _limits_ptrs(self):
        if self._xmin is None:
            return None, None, 1.0
        return nat.ptr(self._xmin), nat.ptr(self._xdelta), self._xdeltajac

    def _width(self):
        return 2 * self._n_out + BINS_MAX * self.n_dim

    def _workspace(self):
        ws = self._ws
        if ws.get("key") != self._width():
            ws.clear()
            ws["key"] = self._width()
            self._state_rows(ws, 16)
            ws["hist"] = torch.zeros((self.n_dim, BINS_MAX), dtype=torch.float64, device=self.device)
            ws["sums"] = torch.zeros(2 * self._n_out, dtype=torch.float64, device=self.device)
        if ws.get("rows") != self._rows:  # the launch shape sets the partial-row count
            ws["rows"] = self._rows
            ws["partials"] = torch.zeros(self._rows * self._width(), dtype=torch.float64,
                                         device=self.device)
        return ws

    def _state_rows(self, ws, rows):
        """One float64 device buffer [avg (5 n_out) | flags (2 int32) | history (rows x
        2 n_out)], so that run_integration reads average, flags and the new history rows
        with one copy; ws["avg"], ws["flags"] (element 0 takes the VF_FLAG_* bits) and
        ws["history"] are views of it.  Growing it keeps the contents."""
        k = self._n_out
        state = torch.zeros(5 * k + 1 + rows * 2 * k, dtype=torch.float64, device=self.device)
        old = ws.get("state")
        if old is not None:
            state[: old.numel()] = old
        ws["state"] = state
        ws["avg"] = state[: 5 * k]
        ws["flags"] = state[5 * k: 5 * k + 1].view(torch.int32)
        ws["history"] = state[5 * k + 1:].view(rows, 2 * k)

    def _history_slot(self):
        ws = self._workspace()
        if self._it >= ws["history"].shape[0]:
            self._state_rows(ws, 2 * ws["history"].shape[0])
        return ws

    def _reset_average(self, clear=False):
        """Start a new weighted average: history row 0 makes the iteration-end
        kernels overwrite the average, so the buffer is only cleared on request."""
        if clear:
            self._workspace()["avg"].zero_()
        self._it = 0

    # ---------------------------------------------------------------- sampling
    def _sample(self, n_events, ev_offset, call, integrand_id, params, train, accumulate,
                u_inj=None, ind=None, x=None, w=None, f=None, xjac=None):
        ws = self._workspace()
        xmin, xdelta, xdj = self._limits_ptrs()
        xjac = self.xjac if xjac is None else xjac
        nat.call("vf_sample", self._ALG, self._prec, self._grid_ptr(), self.n_dim, int(n_events),
                 int(ev_offset), float(xjac), xmin, xdelta, float(xdj), nat.ptr(u_inj),
                 self._seed, call, int(integrand_id), nat.ptr(params), int(bool(train)),
                 int(bool(accumulate)), nat.ptr(ws["partials"]), self._rows, nat.ptr(ind),
                 nat.ptr(x), nat.ptr(w), nat.ptr(f), nat.ptr(ws["flags"]), nat.stream_handle())

    def _injected(self, n):
        if self._uniform_source is None:
            return None
        u = self._uniform_source(n, self.n_dim)
        u = torch.as_tensor(u, dtype=torch.float64, device=self.device).contiguous()
        if tuple(u.shape) != (n, self.n_dim):
            raise ValueError(f"uniform source returned shape {tuple(u.shape)}, expected {(n, self.n_dim)}")
        return u

    def _fill_partials(self, train, n_events=None):
        """All events of one iteration (or the first ``n_events`` of one, weighted
        as part of the whole iteration) into the block-partial rows."""
        self._require_gpu()
        if self.event is None:
            raise RuntimeError("Compile must be ran before running any iterations")
        call = self._next_call()
        n = self.n_events if n_events is None else int(n_events)
        if self._kind == "device":
            self._apply_shape()
            if self._uniform_source is None:
                self._sample(n, 0, call, self._int_id, self._params_dev, train, False)
            else:
                off = 0
                for i, nc in enumerate(_chunk_sizes(n, self.events_per_run)):
                    self._sample(nc, off, call, self._int_id, self._params_dev, train, i > 0,
                                 u_inj=self._injected(nc))
                    off += nc
        else:
            off = 0
            for i, nc in enumerate(_chunk_sizes(n, self.events_per_run)):
                self._torch_chunk(nc, off, call, train, accumulate=i > 0)
                off += nc

    def _chunk_buffers(self, nc):
        ws = self._workspace()
        cap = ws.get("xbuf").shape[0] if "xbuf" in ws else 0
        if cap < nc:
            ws["xbuf"] = torch.empty((nc, self.n_dim), dtype=self._rdtype, device=self.device)
            ws["wbuf"] = torch.empty(nc, dtype=self._rdtype, device=self.device)
            ws["ibuf"] = torch.empty((nc, self.n_dim), dtype=torch.int32, device=self.device)
        return ws["xbuf"][:nc], ws["wbuf"][:nc], ws["ibuf"][:nc]

    def _torch_chunk(self, nc, ev_offset, call, train, accumulate):
        """Unfused path: sampler writes x, w, ind; torch evaluates; a kernel reduces."""
        x, w, ind = self._chunk_buffers(nc)
        self._sample(nc, ev_offset, call, nat.VF_INT_NONE, None, False, False,
                     u_inj=self._injected(nc), ind=ind if self._ALG == nat.VF_ALG_VEGAS else None,
                     x=x, w=w)
        f = self._tf_integrand(x, weight=w)
        f = torch.as_tensor(f).to(device=self.device, dtype=self._rdtype).reshape(nc, -1).contiguous()
        ws = self._workspace()
        nat.call("vf_reduce_events", self._prec, nat.ptr(f), nat.ptr(w),
                 nat.ptr(ind) if self._ALG == nat.VF_ALG_VEGAS else None, int(nc), self.n_dim,
                 self._n_out, int(getattr(self, "_main_dimension", 0)), int(bool(train)),
                 int(bool(accumulate)), nat.ptr(ws["partials"]), self._rows, nat.ptr(ws["flags"]),
                 nat.stream_handle())

    def _end_iteration(self, train, n_events=None, want_hist=False, want_sums=False):
        """Iteration-end kernel; returns (res, sigma) device views of the history row."""
        ws = self._history_slot()
        n = float(self.n_events if n_events is None else n_events)
        # the fp32 form refines its grid in float32 (the reference's float32 arithmetic)
        mode = (2 if self._prec == nat.VF_PREC_F32 else 1) if train else 0
        nat.call("vf_iteration_end", nat.ptr(ws["partials"]), self._rows, self.n_dim, self._n_out,
                 mode, n, float(ALPHA), self._grid_ptr(),
                 nat.ptr(ws["hist"]) if want_hist else None, nat.ptr(ws["sums"]) if want_sums else None,
                 nat.ptr(ws["history"]), nat.ptr(ws["avg"]), int(self._it), nat.ptr(ws["flags"]),
                 nat.stream_handle())
        row = ws["history"][self._it]
        self._it += 1
        k = self._n_out
        if self._vectorial:
            return row[:k], row[k:]
        return row[0], row[1]

    def run_event(self, tensorize_events=False, **kwargs):
        """Run all events of one iteration; returns the accumulated (res, res2[,
        arr_res2]) as device tensors (monte_carlo.py:420-480)."""
        if self._differentiable and self._kind == "torch":
            return self._run_event_autograd()
        return self._event_sums(self.n_events)

    def _event_sums(self, n_events):
        """(res, res2[, arr_res2]) of ``n_events`` events of an iteration, without
        touching the grid or the running average."""
        want_hist = self._ALG == nat.VF_ALG_VEGAS and self._train_now()
        self._fill_partials(train=want_hist, n_events=n_events)
        ws = self._history_slot()
        saved = self._it
        # a scratch history slot so the running average is left untouched
        nat.call("vf_iteration_end", nat.ptr(ws["partials"]), self._rows, self.n_dim, self._n_out, 0,
                 float(self.n_events), float(ALPHA), self._grid_ptr(),
                 nat.ptr(ws["hist"]) if want_hist else None, nat.ptr(ws["sums"]),
                 nat.ptr(ws["history"]), nat.ptr(torch.zeros_like(ws["avg"])), int(saved),
                 nat.ptr(ws["flags"]), nat.stream_handle())
        k = self._n_out
        res = ws["sums"][:k].clone()
        res2 = ws["sums"][k:].clone()
        if not self._vectorial:
            res, res2 = res[0], res2[0]
        if want_hist:
            return res, res2, ws["hist"].clone()
        return res, res2

    # ---------------------------------------------------------------- random numbers
    def generate_random_array(self, n_events, *args):
        """(x, p(x)) for ``n_events`` points (monte_carlo.py:229-247): one
        sampler launch writing x and w (no bin indices) to HBM.  The
        reference's normalisation ``xjac_raw / (xjac n_events)`` is folded into
        the sampler's weight constant (the Jacobian it is given), so that w is
        written once, already normalised."""
        rnds, p, *extra = self._generate_random_array(n_events, *args, want_ind=False,
                                                      xjac=self.xjac / (self.xjac * n_events))
        return rnds, p

    def _generate_random_array(self, n_events, *args, want_ind=True, xjac=None):
        """(x, w[, ind]) of ``n_events`` points, weighted as part of an
        ``self.n_events`` iteration (monte_carlo.py:249-275), or with the
        Jacobian ``xjac`` instead of ``self.xjac``."""
        self._require_gpu()
        n = int(n_events)
        x = torch.empty((n, self.n_dim), dtype=self._rdtype, device=self.device)
        w = torch.empty(n, dtype=self._rdtype, device=self.device)
        ind = torch.empty((n, self.n_dim), dtype=torch.int32, device=self.device) \
            if self._ALG == nat.VF_ALG_VEGAS and want_ind else None
        self._sample(n, 0, self._next_call(), nat.VF_INT_NONE, None, False, False,
                     u_inj=self._injected(n), ind=ind, x=x, w=w, xjac=xjac)
        if ind is None:
            return x, w
        return x, w, ind

    # ---------------------------------------------------------------- compile
    def trace(self, n_events=50):
        rnds, wgt, *_ = self._generate_random_array(n_events)
        if self._kind == "torch":
            self._tf_integrand(rnds, weight=wgt)

    def compile(self, integrand, compilable=True, signature=None, trace=False, check=True):
        """Register the integrand (monte_carlo.py:489-636).

        ``integrand`` is either a ``DeviceIntegrand`` (evaluated inside the
        sampler kernel) or a callable on torch tensors ``f(xarr[, weight][,
        n_dim])`` returning ``(n,)`` or, for VegasFlow/PlainFlow, ``(n, k)``.
        ``compilable`` and ``signature`` are accepted for compatibility (there is
        no tracing compiler); ``check`` runs the reference's 23-event shape check
        on torch callables."""
        kwargs = {"compilable": compilable, "signature": signature, "trace": trace}
        self._compilation_arguments = (integrand, kwargs)
        self._integrand = integrand
        self._vectorial = False
        self._n_out = 1
        if isinstance(integrand, DeviceIntegrand):
            integrand.check_dims(self.n_dim)
            self._kind = "device"
            self._int_id = integrand.integrand_id
            if getattr(integrand, "source", None) is not None:  # CUDA source: NVRTC on first use
                if self.device.type == "cuda":
                    self._int_id = self._compile_cuda_integrand(integrand)
            self._params_host = integrand.params(self.n_dim)
            self._params_dev = torch.as_tensor(self._params_host, dtype=torch.float64,
                                               device=self.device) if self.device.type == "cuda" else None
            self._tf_integrand = integrand
        else:
            if not callable(integrand):
                raise TypeError("the integrand must be callable or a DeviceIntegrand")
            self._kind = "torch"
            try:
                args = inspect.getfullargspec(integrand).args[1:]
            except TypeError:
                args = []
            n_dim = self.n_dim

            def new_integrand(xarr, weight=None, **kw):
                if "weight" in args and "n_dim" in args:
                    return integrand(xarr, n_dim=n_dim, weight=weight, **kw)
                if "weight" in args:
                    return integrand(xarr, weight=weight, **kw)
                if "n_dim" in args:
                    return integrand(xarr, n_dim=n_dim, **kw)
                return integrand(xarr, **kw)

            self._tf_integrand = new_integrand
            if check:
                event_size = 23
                test_array = torch.rand((event_size, self.n_dim), dtype=self._rdtype, device=self.device)
                wgt = torch.rand(event_size, dtype=self._rdtype, device=self.device)
                res_tmp = torch.as_tensor(new_integrand(test_array, weight=wgt))
                res_shape = tuple(res_tmp.shape)
                expected_shape = (event_size,)
                if len(res_shape) == 2:
                    self._vectorial = True
                    expected_shape = tuple(res_tmp.reshape(event_size, -1).shape)
                    if not self._can_run_vectorial(expected_shape):
                        raise NotImplementedError(
                            f"The {self.__class__.__name__} algorithm does not support vectorial "
                            "integrands")
                    self._n_out = expected_shape[1]
                if res_shape != expected_shape:
                    error_str = "the shape of the integrand output should be: (n_events,"
                    if self._vectorial:
                        error_str += " output_dim,"
                    logger.error(f"Wrong integrand output shape, {error_str})")
                    raise ValueError(
                        "The integrand is not returning a value per event, expected shape: "
                        f"{expected_shape}, found: {res_shape}")
        self.event = self._fill_partials
        if self.device.type == "cuda":
            self._choose_rows()
            self._ws.clear()
            if self._autotune:
                self.tune_launch()
        if trace:
            self.trace(n_events=23)

    def _compile_cuda_integrand(self, integrand):
        return integrand.compile_for(self._ALG, self._prec, self.n_dim)

    # ---------------------------------------------------------------- launch shape
    @property
    def launch_shape(self):
        """The fp32 sampler launch shape this integrator uses (``None`` = default)."""
        return self._shape

    def set_launch_shape(self, shape):
        """Use ``shape`` (an ``autotune.LaunchShape`` or ``None`` for the default)
        for this integrator's fused fp32 sampler launches."""
        self._shape = shape
        if self.device.type == "cuda" and self.event is not None:
            self._choose_rows()

    def tune_launch(self, force=False):
        """Time the candidate launch shapes on this workload (or read the cached
        winner) and use the fastest; returns it, or ``None`` where the
        configuration has no launch shape to choose (not fused fp32 VEGAS)."""
        shape = autotune.tune(self, force=force)
        if shape is not None:
            self.set_launch_shape(shape)
        return shape

    def _apply_shape(self):
        if autotune.fused_f32(self):
            autotune.ensure(self._shape or autotune.DEFAULT_SHAPE)

    def _choose_rows(self):
        lib = nat.load()
        import ctypes
        self._apply_shape()
        rows = ctypes.c_int(0)
        integ = self._int_id if self._kind == "device" else nat.VF_INT_SYMGAUSS
        nat.check(lib.vf_sample_rows(self._ALG, self._prec, self.n_dim, integ, 1, ctypes.byref(rows)))
        # a small iteration launches no more blocks than give every thread a few
        # events: idle blocks still stage the table, clear and read back their
        # histogram, and add partial rows for the iteration end to reduce
        n = self.n_events
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        spread = min(sms, -(-n // EVENTS_PER_BLOCK_MIN))
        self._rows = max(1, min(rows.value, max(spread, -(-n // EVENTS_PER_BLOCK_TARGET))))

    def _recompile(self):
        if self._compilation_arguments is None:
            raise RuntimeError("recompile was called without ever having called compile")
        self.compile(self._compilation_arguments[0], **self._compilation_arguments[1])

    # ---------------------------------------------------------------- integration
    # ---------------------------------------------------------------- CUDA-graph iterations
    def _graph_ready(self, histograms):
        return (self._cuda_graph and self._GRAPH_ITERATIONS and self._kind == "device" and not histograms
                and self._uniform_source is None and self.device.type == "cuda")

    def _graph_call(self, ws):
        xmin, xdelta, xdj = self._limits_ptrs()
        nat.call("vf_iteration_dev", self._ALG, self._prec, self._grid_ptr(), self.n_dim, int(self.n_events),
                 float(self.xjac), xmin, xdelta, float(xdj), self._seed, nat.ptr(ws["counters"][0:1]),
                 nat.ptr(ws["counters"][1:2]), int(self._int_id), nat.ptr(self._params_dev),
                 int(bool(self._train_now())), float(ALPHA), nat.ptr(ws["partials"]), self._rows,
                 nat.ptr(ws["history"]), int(ws["history"].shape[0]), nat.ptr(ws["avg"]), nat.ptr(ws["flags"]),
                 nat.stream_handle())

    def _graph_signature(self, ws):
        """Every value the captured call was made with: a change means a new capture."""
        def addr(p):
            return p.value if p is not None else 0

        xmin, xdelta, xdj = self._limits_ptrs()
        return (self._ALG, self._prec, addr(self._grid_ptr()), self.n_events, self.xjac, self._seed, self._int_id,
                self._params_dev.data_ptr(), bool(self._train_now()), self._rows, ws["partials"].data_ptr(),
                ws["history"].data_ptr(), ws["history"].shape[0], ws["avg"].data_ptr(), ws["flags"].data_ptr(),
                ws["counters"].data_ptr(), addr(xmin), addr(xdelta), xdj, self._shape)

    def _capture(self, ws, unroll):
        """A CUDA graph of ``unroll`` consecutive iteration calls."""
        from .utils import capture_guard, preload_kernels
        preload_kernels(self.device)
        torch.cuda.synchronize(self.device)
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        with capture_guard(), torch.cuda.stream(side):
            with torch.cuda.graph(g, stream=side):
                for _ in range(unroll):
                    self._graph_call(ws)
        torch.cuda.current_stream(self.device).wait_stream(side)
        return g

    def _graph_for(self, n_iter, unroll=1):
        """The CUDA graph of ``unroll`` iterations (captured again whenever an
        argument of the captured call changed), with room for ``n_iter``
        history rows.  ``self._graph`` is the one-iteration graph; graphs of
        several iterations are kept beside it for the same arguments."""
        ws = self._workspace()
        if ws["history"].shape[0] < n_iter:
            self._state_rows(ws, max(n_iter, 2 * ws["history"].shape[0]))
        if "counters" not in ws:
            ws["counters"] = torch.zeros(2, dtype=torch.int32, device=self.device)
        self._apply_shape()
        key = self._graph_signature(ws)
        if self._graph is None or self._graph_key != key:
            self._graph, self._graph_key = self._capture(ws, 1), key
            self._graphs_unrolled = {}
        if unroll == 1:
            return self._graph, ws
        g = self._graphs_unrolled.get(unroll)
        if g is None:
            g = self._graphs_unrolled[unroll] = self._capture(ws, unroll)
        return g, ws

    def _run_graph(self, n_iter, log_time):
        """``n_iter`` iterations as replays of captured iterations: the Philox
        call counter and the history row advance on the device.  Without
        per-iteration logging, up to GRAPH_UNROLL iterations go into one replay
        (one graph launch, and one host call, instead of several)."""
        unroll = 1 if self._verbose else max(1, min(n_iter, GRAPH_UNROLL))
        g1, ws = self._graph_for(n_iter)
        gu = self._graph_for(n_iter, unroll)[0] if unroll > 1 else g1
        # the start counters (call, iteration) as one 64-bit device fill: asynchronous,
        # and no pinned host buffer (whose release could record events on a stream
        # while another stream captures)
        start = np.array([self._call_ctr & 0xFFFFFFFF, self._it], dtype=np.uint32).view(np.int64)
        ws["counters"].view(torch.int64).fill_(int(start[0]))
        if self._verbose:
            for i in range(n_iter):
                t0 = time.time()
                g1.replay()
                self._history.append([None, None, None])
                row = ws["history"][self._it + i].cpu().numpy()
                time_str = f"(took {time.time() - t0:.5f} s)" if log_time else ""
                logger.info(print_iteration(i, float(row[0]), float(row[1]), extra=time_str))
        else:
            full, rest = divmod(n_iter, unroll)
            for _ in range(full):
                gu.replay()
            for _ in range(rest):
                g1.replay()
            self._history.extend([None, None, None] for _ in range(n_iter))
        self._call_ctr += n_iter
        self._it += n_iter

    def run_integration(self, n_iter, log_time=True, histograms=None):
        """Run ``n_iter`` iterations; returns (result, sigma) (monte_carlo.py:645-741).

        With ``cuda_graph=True`` (device integrands; VegasFlow, PlainFlow and
        VegasFlowPlus) the iterations are replays of one captured CUDA graph (two
        kernels, no host work between iterations)."""
        self._require_gpu()
        self._reset_average(clear=n_iter < 1)
        first = len(self._history)
        all_results = []
        graph = self._graph_ready(histograms)
        if graph:
            with _nvtx(f"vegasflow: {n_iter} graph iterations"):
                self._run_graph(n_iter, log_time)
        for i in range(0 if graph else n_iter):
            if log_time:
                start = time.time()
            with _nvtx(f"vegasflow: iteration {i}"):
                res, error = self._run_iteration()
            all_results.append((res, error))
            hist_copy = copy.deepcopy(histograms) if histograms else None
            if histograms:
                for h in histograms:
                    h.zero_()
            self._history.append([res, error, hist_copy])
            if self._verbose:
                torch.cuda.current_stream().synchronize()
                time_str = f"(took {time.time() - start:.5f} s)" if log_time else ""
                if self._vectorial:
                    info = [print_iteration(i, float(rr), float(ee), extra=f" [dimension {d}] {time_str}")
                            for d, (rr, ee) in enumerate(zip(res.tolist(), error.tolist()))]
                else:
                    info = [print_iteration(i, float(res), float(error), extra=time_str)]
                logger.info("\n      ".join(info))
        ws = self._workspace()
        # one copy of average, flags word (its bits carried through a float64 slot,
        # which the copy moves without arithmetic) and history rows
        k = self._n_out
        host = ws["state"][: 5 * k + 1 + self._it * 2 * k].cpu().numpy()
        avg = host[: 5 * k].reshape(k, 5)
        flags = int(host[5 * k: 5 * k + 1].view(np.int32)[0])
        hist_rows = host[5 * k + 1:].reshape(self._it, 2 * k)
        self._check_flags(flags)
        base = self._it - n_iter
        for i in range(n_iter):
            r, s = hist_rows[base + i][:k], hist_rows[base + i][k:]
            self._history[first + i][0] = r.copy() if self._vectorial else np.float64(r[0])
            self._history[first + i][1] = s.copy() if self._vectorial else np.float64(s[0])
            self._history[first + i] = tuple(self._history[first + i])
        if histograms:
            weight_sum = 0.0
            for h in histograms:
                h.zero_()
            for i in range(n_iter):
                wgt = 1.0 / np.power(self._history[first + i][1], 2)
                weight_sum += wgt
                for aux_h, curr_h in zip(histograms, self._history[first + i][2]):
                    aux_h.add_(curr_h * float(np.mean(wgt)))
            for h in histograms:
                h.div_(float(np.mean(weight_sum)))
        self.chi2_dof = avg[:, 4].copy() if self._vectorial else float(avg[0, 4])
        if self._vectorial:
            final_result, sigma = avg[:, 2].copy(), avg[:, 3].copy()
            if self._verbose:
                logger.info("\n     ".join(f"Final results [dim = {d}]: {rr:g} +/- {ee:g}"
                                           for d, (rr, ee) in enumerate(zip(final_result, sigma))))
        else:
            final_result, sigma = np.float64(avg[0, 2]), np.float64(avg[0, 3])
            if self._verbose:
                logger.info(f" > Final results: {final_result:g} +/- {sigma:g}")
        return final_result, sigma

    def _check_flags(self, flags):
        if flags & nat.VF_FLAG_INDEX_RANGE:
            logger.warning("some uniforms mapped outside the grid and were clamped (injected "
                           "uniforms outside [0, 1)?)")
        if flags & nat.VF_FLAG_REFINE_OVERRUN:
            logger.warning("grid refinement walked past the last bin (rounding); clamped")
        if flags & nat.VF_FLAG_NONFINITE:
            logger.warning("a partial sum was NaN or Inf")
        if flags:
            self._workspace()["flags"].zero_()
        if flags & nat.VF_FLAG_TIMEOUT:
            raise nat.VegasGB300Error(nat.VF_ERR_TIMEOUT, "a device-side copy of injected uniforms never "
                                      "completed; the iteration's sums are incomplete")

    def make_differentiable(self):
        """monte_carlo.py:389-418: returns ``run_event``, whose results then
        follow torch autograd.  For a torch-callable integrand the events' x and
        w come from the sampler (they depend on no parameter) and the sums over
        events are taken by torch, so ``run_event()[0]`` is connected to the
        integrand's autograd graph: gradients with respect to the integrand's
        parameters flow through the integral, and each call draws new events.
        Device integrands have fixed parameters; their results carry no graph."""
        if self.distribute:
            raise ValueError("Differentiation is not compatible with distribution")
        self._differentiable = True
        if self.event is not None:
            logger.warning("Recompiling...")
            self._recompile()
        return self.run_event

    def _run_event_autograd(self):
        """run_event for a torch integrand with the sums taken by torch:
        (res, res2[, arr_res2]) with res and res2 in the autograd graph."""
        self._require_gpu()
        vegas = self._ALG == nat.VF_ALG_VEGAS
        want_hist = vegas and self._train_now()
        call = self._next_call()
        res = res2 = hist = None
        off = 0
        for nc in _chunk_sizes(self.n_events, self.events_per_run):
            # fresh buffers: the graph keeps x and w for the backward pass
            x = torch.empty((nc, self.n_dim), dtype=self._rdtype, device=self.device)
            w = torch.empty(nc, dtype=self._rdtype, device=self.device)
            ind = torch.empty((nc, self.n_dim), dtype=torch.int32, device=self.device) if vegas else None
            self._sample(nc, off, call, nat.VF_INT_NONE, None, False, False, u_inj=self._injected(nc), ind=ind,
                         x=x, w=w)
            f = torch.as_tensor(self._tf_integrand(x, weight=w)).to(device=self.device)
            tmp = (w.reshape(nc, 1) * f.reshape(nc, -1)) if self._vectorial else w * f.reshape(nc)
            r, r2 = tmp.sum(0), (tmp * tmp).sum(0)
            res = r if res is None else res + r
            res2 = r2 if res2 is None else res2 + r2
            if want_hist:
                from .utils import consume_array_into_indices
                main = tmp[:, getattr(self, "_main_dimension", 0)] if self._vectorial else tmp
                t2 = (main * main).detach().to(torch.float64)
                h = torch.stack([consume_array_into_indices(t2, ind[:, j:j + 1], BINS_MAX)
                                 for j in range(self.n_dim)])
                hist = h if hist is None else hist + h
            off += nc
        if want_hist:
            return res, res2, hist
        return res, res2

    # ---------------------------------------------------------------- device pool
    def get_device(self):
        """The first free device of the pool, now taken, or None (monte_carlo.py:318-332);
        the pool is this integrator's GPU."""
        with self.lock:
            if self.devices is None:
                self.devices = {self.device: True}
            for device, available in self.devices.items():
                if available:
                    self.devices[device] = False
                    return device
        return None

    def release_device(self, device):
        """Makes ``device`` available again (monte_carlo.py:334-340)."""
        with self.lock:
            if self.devices is None:
                self.devices = {}
            self.devices[device] = True

    def device_run(self, ncalls, sent_pc=100.0, **kwargs):
        """The accumulables (res, res2[, arr_res2]) of ``ncalls`` events, weighted as
        part of an ``n_events`` iteration, on the pool's device (monte_carlo.py:342-365)."""
        if self._verbose:
            print(f"Events sent to the computing device: {sent_pc:.1f} %", end="\r")
        if not self.event:
            raise RuntimeError("Compile must be ran before running any iterations")
        device = self.get_device()
        try:
            if self._differentiable and self._kind == "torch" and int(ncalls) == self.n_events:
                return self._run_event_autograd()
            return self._event_sums(int(ncalls))
        finally:
            if device is not None:
                self.release_device(device)

    def set_distribute(self, queue_object):
        raise NotImplementedError("dask distribution is not part of the GB300 build (one GPU)")


def wrapper(integrator_class, integrand, n_dim, n_iter, total_n_events, compilable=True, **kwargs):
    """monte_carlo.py:744-762."""
    mc_instance = integrator_class(n_dim, total_n_events, **kwargs)
    mc_instance.compile(integrand, compilable=compilable)
    return mc_instance.run_integration(n_iter)


def sampler(integrator_class, integrand, n_dim, total_n_events, training_steps=5, compilable=True,
            return_class=False, **kwargs):
    """monte_carlo.py:765-794."""
    mc_instance = integrator_class(n_dim, total_n_events, verbose=False, **kwargs)
    mc_instance.compile(integrand, compilable=compilable)
    _ = mc_instance.run_integration(training_steps, log_time=False)
    if return_class:
        return mc_instance
    return mc_instance.generate_random_array
