"""VegasFlowPlus: VEGAS+ importance + adaptive stratified sampling
(vegasflow vflowplus.py:83-282).

Device state: the VEGAS grid, ``n_ev`` (events per hypercube, int32) and its
exclusive prefix sum ``ev_start`` (int64, n_hypercubes + 1 entries).  One
sampler launch and one iteration-end launch per iteration; the adaptive
reallocation (``redistribute_samples``) runs inside the iteration-end kernel,
so the event count of the next iteration never round-trips through the host
for device integrands.
"""

from __future__ import annotations

import logging

import numpy as np
import torch

from . import _native as nat
from .configflow import ALPHA, BETA, BINS_MAX, MAX_NEVAL_HCUBE
from .monte_carlo import sampler, wrapper
from .vflow import VegasFlow

logger = logging.getLogger("vegasflow.vflowplus")


def stratification(n_dim, n_events, adaptive):
    """vflowplus.py:105-139: (adaptive, n_strat, n_hypercubes, min_neval, n_events).

    The powers are float32, as TensorFlow evaluates ``tf.math.pow`` on Python
    floats (vflowplus.py:115-121)."""
    if n_dim > 13 and adaptive:
        adaptive = False
        logger.warning("Disabling adaptive mode from VegasFlowPlus, too many dimensions!")
    neval_eff = int(n_events / 2) if adaptive else int(n_events)
    n_strat = np.floor(np.power(np.float32(neval_eff / 2), np.float32(1 / n_dim)))
    if np.power(np.float32(n_strat), np.float32(n_dim)) > MAX_NEVAL_HCUBE:
        n_strat = np.floor(np.power(np.float32(1e4), np.float32(1 / n_dim)))
    n_strat = int(n_strat)
    n_hcubes = n_strat ** n_dim
    min_neval = max(int(neval_eff // n_hcubes), 2)
    return adaptive, n_strat, n_hcubes, min_neval, min_neval * n_hcubes


class VegasFlowPlus(VegasFlow):
    """VEGAS+ (vflowplus.py:83)."""

    _FUSED_F32_SAMPLER = False  # samples per hypercube through its own kernels
    _GRAPH_ITERATIONS = True  # one iteration is vf_plus_iteration_dev (CUDA-graph replayable)

    def __init__(self, n_dim, n_events, train=True, adaptive=False, events_limit=None, **kwargs):
        if events_limit is None:  # vflowplus.py:89-99
            logger.info("Events per device limit set to %d", n_events)
            events_limit = n_events
        elif events_limit < n_events:
            logger.warning("VegasFlowPlus needs to hold all events in memory at once, "
                           "setting the `events_limit` to be equal to `n_events=%d`", n_events)
            events_limit = n_events
        super().__init__(n_dim, n_events, train, events_limit=events_limit, **kwargs)
        self._init_calls = int(n_events)
        (self._adaptive, self._n_strat, n_hcubes, self.min_neval_hcube,
         n_tot) = stratification(n_dim, n_events, adaptive)
        self._n_hcubes = n_hcubes
        self._n_events = n_tot
        self._modified_jac = 1.0 / n_hcubes
        self._n_ev_stale = False
        self.n_ev = torch.full((n_hcubes,), self.min_neval_hcube, dtype=torch.int32, device=self.device)
        self._ev_start = torch.arange(n_hcubes + 1, dtype=torch.int64,
                                      device=self.device) * self.min_neval_hcube
        if self._adaptive:
            logger.warning("Variable number of events requires function signatures all across")

    # ---------------------------------------------------------------- properties
    @property
    def xjac(self):
        return self._modified_jac

    @property
    def n_events(self):
        if self._n_ev_stale:
            self._n_events = int(self._ev_start[-1].item())
            self._n_ev_stale = False
        return self._n_events

    @n_events.setter
    def n_events(self, val):
        self._n_events = int(val)
        self._n_ev_stale = False
        self.events_per_run = self._events_limit
        self._recompile()

    @property
    def n_hypercubes(self):
        return self._n_hcubes

    def _can_run_vectorial(self, expected_shape=None):
        super()._can_run_vectorial(expected_shape)
        return False

    def _run_event_autograd(self):
        """(ress, arr_var[, arr_res2]) of one iteration's events with the
        per-hypercube sums taken by torch (vflowplus.py:187-220), so that they
        follow the integrand's autograd graph."""
        self._require_gpu()
        ws = self._plus_buffers()
        call = self._next_call()
        xmin, xdelta, xdj = self._limits_ptrs()
        n_total = self.n_events
        u = self._injected(n_total)
        x = torch.empty((n_total, self.n_dim), dtype=self._rdtype, device=self.device)
        w = torch.empty(n_total, dtype=self._rdtype, device=self.device)
        ind = torch.empty((n_total, self.n_dim), dtype=torch.int32, device=self.device)
        nat.call("vf_plus_sample", self._prec, nat.ptr(self.divisions), self.n_dim, self._n_strat,
                 self._n_hcubes, nat.ptr(self.n_ev), nat.ptr(self._ev_start), float(self.xjac), xmin,
                 xdelta, float(xdj), nat.ptr(u), self._seed, call, nat.VF_INT_NONE, None, 0, None,
                 None, None, self._rows, nat.ptr(ind), nat.ptr(x), nat.ptr(w), nat.ptr(ws["flags"]),
                 nat.stream_handle())
        f = torch.as_tensor(self._tf_integrand(x, weight=w)).to(device=self.device).reshape(-1)
        tmp = w * f
        n_ev = self.n_ev.to(torch.int64)
        segm = torch.repeat_interleave(torch.arange(self._n_hcubes, device=self.device), n_ev,
                                       output_size=n_total)  # vflowplus.py:67 (events laid out by hypercube)
        zeros = torch.zeros(self._n_hcubes, dtype=tmp.dtype, device=self.device)
        ress = zeros.index_add(0, segm, tmp)
        ress2 = zeros.index_add(0, segm, tmp * tmp)
        arr_var = ress2 * n_ev.to(tmp.dtype) - ress * ress
        if not self.train:
            return ress, arr_var
        from .utils import consume_array_into_indices
        t2 = (tmp * tmp).detach().to(torch.float64)
        hist = torch.stack([consume_array_into_indices(t2, ind[:, j:j + 1], BINS_MAX) for j in range(self.n_dim)])
        return ress, arr_var, hist

    # ---------------------------------------------------------------- VEGAS+ steps
    def redistribute_samples(self, arr_var):
        """vflowplus.py:153-163 on the device: new ``n_ev`` from the per-hypercube
        variances, then the event count."""
        var = torch.as_tensor(arr_var, dtype=torch.float64, device=self.device)
        damped = torch.pow(var, BETA / 2)
        new = torch.fmax(torch.full_like(damped, float(self.min_neval_hcube)),
                         damped * float(self._init_calls) / 2 / torch.sum(damped))
        self.n_ev = new.to(torch.int32)
        self._ev_start[1:] = torch.cumsum(self.n_ev.to(torch.int64), 0)
        self._ev_start[0] = 0
        self._n_ev_stale = True

    def _compile_cuda_integrand(self, integrand):
        """NVRTC-compile the user's device function into the VEGAS+ samplers."""
        return integrand.compile_for(nat.VF_ALG_PLUS, self._prec, self.n_dim)

    def _plus_rows(self):
        import ctypes
        rows = ctypes.c_int(0)
        nat.check(nat.load().vf_plus_rows(self._prec, self.n_dim, self._n_hcubes, ctypes.byref(rows)))
        return rows.value

    def _choose_rows(self):
        self._rows = self._plus_rows()

    def _plus_buffers(self):
        ws = self._workspace()
        if "ress" not in ws:
            ws["ress"] = torch.zeros(self._n_hcubes, dtype=torch.float64, device=self.device)
            ws["ress2"] = torch.zeros(self._n_hcubes, dtype=torch.float64, device=self.device)
            ws["arr_var"] = torch.zeros(self._n_hcubes, dtype=torch.float64, device=self.device)
        return ws

    def _fill_plus(self, train):
        self._require_gpu()
        if self.event is None:
            raise RuntimeError("Compile must be ran before running any iterations")
        ws = self._plus_buffers()
        call = self._next_call()
        xmin, xdelta, xdj = self._limits_ptrs()
        n_total = None
        u = None
        if self._uniform_source is not None or self._kind == "torch":
            n_total = self.n_events  # synchronises when the device reallocated
            u = self._injected(n_total)
        if self._kind == "device":
            nat.call("vf_plus_sample", self._prec, nat.ptr(self.divisions), self.n_dim, self._n_strat,
                     self._n_hcubes, nat.ptr(self.n_ev), nat.ptr(self._ev_start), float(self.xjac), xmin,
                     xdelta, float(xdj), nat.ptr(u), self._seed, call, self._int_id,
                     nat.ptr(self._params_dev), int(bool(train)), nat.ptr(ws["ress"]), nat.ptr(ws["ress2"]),
                     nat.ptr(ws["partials"]), self._rows, None, None, None, nat.ptr(ws["flags"]),
                     nat.stream_handle())
        else:
            x = torch.empty((n_total, self.n_dim), dtype=self._rdtype, device=self.device)
            w = torch.empty(n_total, dtype=self._rdtype, device=self.device)
            ind = torch.empty((n_total, self.n_dim), dtype=torch.int32, device=self.device)
            nat.call("vf_plus_sample", self._prec, nat.ptr(self.divisions), self.n_dim, self._n_strat,
                     self._n_hcubes, nat.ptr(self.n_ev), nat.ptr(self._ev_start), float(self.xjac), xmin,
                     xdelta, float(xdj), nat.ptr(u), self._seed, call, nat.VF_INT_NONE, None, 0, None,
                     None, None, self._rows, nat.ptr(ind), nat.ptr(x), nat.ptr(w), nat.ptr(ws["flags"]),
                     nat.stream_handle())
            f = self._tf_integrand(x, weight=w)
            f = torch.as_tensor(f).to(device=self.device, dtype=self._rdtype).reshape(-1).contiguous()
            nat.call("vf_plus_reduce_events", self._prec, nat.ptr(f), nat.ptr(w), nat.ptr(ind),
                     nat.ptr(self.n_ev), nat.ptr(self._ev_start), self.n_dim, self._n_hcubes,
                     int(bool(train)), nat.ptr(ws["ress"]), nat.ptr(ws["ress2"]), nat.ptr(ws["partials"]),
                     self._rows, nat.stream_handle())

    def _end_plus(self, train, want_hist=False):
        ws = self._history_slot()
        ws = self._plus_buffers()
        nat.call("vf_plus_iteration_end", nat.ptr(ws["ress"]), nat.ptr(ws["ress2"]), nat.ptr(self.n_ev),
                 nat.ptr(self._ev_start), self._n_hcubes, int(self._adaptive), int(self.min_neval_hcube),
                 float(self._init_calls), nat.ptr(ws["partials"]), self._rows, self.n_dim,
                 (2 if self._prec == nat.VF_PREC_F32 else 1) if train else 0,  # fp32: float32 refinement
                 float(ALPHA), float(BETA), nat.ptr(self.divisions),
                 nat.ptr(ws["hist"]) if want_hist else None, nat.ptr(ws["arr_var"]), nat.ptr(ws["history"]),
                 nat.ptr(ws["avg"]), int(self._it), nat.ptr(ws["flags"]), nat.stream_handle())
        if self._adaptive:
            self._n_ev_stale = True
        row = ws["history"][self._it]
        self._it += 1
        return row[0], row[1]

    # ---------------------------------------------------------------- CUDA-graph iterations
    def _graph_signature(self, ws):
        def addr(p):
            return p.value if p is not None else 0

        ws = self._plus_buffers()  # allocated before any capture
        xmin, xdelta, xdj = self._limits_ptrs()
        return ("plus", self._prec, self.divisions.data_ptr(), self.n_ev.data_ptr(), self._ev_start.data_ptr(),
                self.xjac, self._seed, self._int_id, self._params_dev.data_ptr(), bool(self.train), self._adaptive,
                self._rows, ws["partials"].data_ptr(), ws["ress"].data_ptr(), ws["ress2"].data_ptr(),
                ws["history"].data_ptr(), ws["history"].shape[0], ws["avg"].data_ptr(), ws["flags"].data_ptr(),
                ws["counters"].data_ptr(), addr(xmin), addr(xdelta), xdj)

    def _graph_call(self, ws):
        ws = self._plus_buffers()
        xmin, xdelta, xdj = self._limits_ptrs()
        nat.call("vf_plus_iteration_dev", self._prec, nat.ptr(self.divisions), self.n_dim, self._n_strat,
                 self._n_hcubes, nat.ptr(self.n_ev), nat.ptr(self._ev_start), float(self.xjac), xmin, xdelta,
                 float(xdj), self._seed, nat.ptr(ws["counters"][0:1]), nat.ptr(ws["counters"][1:2]),
                 int(self._int_id), nat.ptr(self._params_dev), int(bool(self.train)), int(self._adaptive),
                 int(self.min_neval_hcube), float(self._init_calls), float(ALPHA), float(BETA),
                 nat.ptr(ws["ress"]), nat.ptr(ws["ress2"]), nat.ptr(ws["partials"]), self._rows,
                 nat.ptr(ws["history"]), int(ws["history"].shape[0]), nat.ptr(ws["avg"]), nat.ptr(ws["flags"]),
                 nat.stream_handle())

    def _run_graph(self, n_iter, log_time):
        super()._run_graph(n_iter, log_time)
        if self._adaptive:
            self._n_ev_stale = True  # the replays reallocated on the device

    def _iteration_content(self):
        """vflowplus.py:222-241: sample, sums, sigma, reallocation, refinement."""
        self._fill_plus(train=self.train)
        return self._end_plus(train=self.train)

    def _run_iteration(self):
        return self._iteration_content()

    def run_event(self, tensorize_events=None, **kwargs):
        """(ress, arr_var, arr_res2) of one iteration's events (vflowplus.py:187-220)
        without updating the grid, the allocation or the running average."""
        if self._differentiable and self._kind == "torch":
            return self._run_event_autograd()
        want_hist = bool(self.train)
        self._fill_plus(train=want_hist)
        ws = self._history_slot()
        adaptive, self._adaptive = self._adaptive, False
        avg_saved = ws["avg"].clone()
        try:
            nat.call("vf_plus_iteration_end", nat.ptr(ws["ress"]), nat.ptr(ws["ress2"]),
                     nat.ptr(self.n_ev), nat.ptr(self._ev_start), self._n_hcubes, 0,
                     int(self.min_neval_hcube), float(self._init_calls), nat.ptr(ws["partials"]), self._rows,
                     self.n_dim, 0, float(ALPHA), float(BETA), None,
                     nat.ptr(ws["hist"]) if want_hist else None, nat.ptr(ws["arr_var"]),
                     nat.ptr(ws["history"]), nat.ptr(ws["avg"]), int(self._it), nat.ptr(ws["flags"]),
                     nat.stream_handle())
        finally:
            self._adaptive = adaptive
        ws["avg"].copy_(avg_saved)
        out = (ws["ress"].clone(), ws["arr_var"].clone())
        if want_hist:
            return out + (ws["hist"].clone(),)
        return out

    def _event_sums(self, n_events):
        # the hypercube allocation covers whole iterations (events_limit = n_events,
        # vflowplus.py:88-100), so a device run is always one
        if int(n_events) != self.n_events:
            raise NotImplementedError(f"VegasFlowPlus runs whole iterations of {self.n_events} events, "
                                      f"not {n_events}")
        return self.run_event()

    def _generate_random_array(self, n_events, *args, want_ind=True, xjac=None):
        """(x, w, ind, segm) of one full iteration's layout (vflowplus.py:165-171);
        (x, w) alone without ``want_ind``; the weights with the Jacobian
        ``xjac`` instead of ``self.xjac`` when it is given."""
        self._require_gpu()
        n = self.n_events
        x = torch.empty((n, self.n_dim), dtype=self._rdtype, device=self.device)
        w = torch.empty(n, dtype=self._rdtype, device=self.device)
        ind = torch.empty((n, self.n_dim), dtype=torch.int32, device=self.device) if want_ind else None
        xmin, xdelta, xdj = self._limits_ptrs()
        u = self._injected(n)
        xjac = self.xjac if xjac is None else xjac
        nat.call("vf_plus_sample", self._prec, nat.ptr(self.divisions), self.n_dim, self._n_strat,
                 self._n_hcubes, nat.ptr(self.n_ev), nat.ptr(self._ev_start), float(xjac), xmin,
                 xdelta, float(xdj), nat.ptr(u), self._seed, self._next_call(), nat.VF_INT_NONE, None, 0,
                 None, None, None, max(1, self._rows or self._plus_rows()), nat.ptr(ind), nat.ptr(x),
                 nat.ptr(w), None, nat.stream_handle())
        if not want_ind:
            return x, w
        segm = torch.repeat_interleave(torch.arange(self._n_hcubes, device=self.device),
                                       self.n_ev.to(torch.int64))
        return x, w, ind, segm

    def generate_random_array(self, n_events, *args):
        """vflowplus.py:173-185: whole iterations concatenated, cut to
        ``n_events``.  The reference's weight normalisation
        ``w_raw / (xjac n_it) * n_it / n_events`` is folded into the sampler's
        Jacobian, so each iteration's weights are written once, normalised."""
        rnds, wgts = [], []
        n_it = self.n_events
        xjac = self.xjac / (self.xjac * n_it) * n_it / n_events
        for _ in range(n_events // n_it + 1):
            r, w, *_ = self._generate_random_array(n_it, want_ind=False, xjac=xjac)
            rnds.append(r)
            wgts.append(w)
        if len(rnds) == 1:
            return rnds[0][:n_events], wgts[0][:n_events]
        return torch.cat(rnds, dim=0)[:n_events], torch.cat(wgts, dim=0)[:n_events]


def vegasflowplus_wrapper(integrand, n_dim, n_iter, total_n_events, **kwargs):
    """Convenience wrapper (vflowplus.py:250-265)."""
    return wrapper(VegasFlowPlus, integrand, n_dim, n_iter, total_n_events, **kwargs)


def vegasflowplus_sampler(*args, **kwargs):
    """Train and return ``generate_random_array`` (vflowplus.py:268-282)."""
    return sampler(VegasFlowPlus, *args, **kwargs)
