"""VegasFlow: VEGAS importance sampling (vegasflow vflow.py:215-481).

The grid ``divisions`` is a (n_dim, 51) float64 device tensor, initialised to
``linspace(0, 1, 51)`` per dimension (vflow.py:239-242) and refined in place
by the iteration-end kernel while ``train`` is on.  ``save_grid`` /
``load_grid`` use the reference's JSON format, so grids move between the two
implementations.
"""

from __future__ import annotations

import json
import logging

import numpy as np
import torch

from . import _native as nat
from .configflow import ALPHA, BINS_MAX
from .monte_carlo import MonteCarloFlow, sampler, wrapper

logger = logging.getLogger("vegasflow.vflow")


class VegasFlow(MonteCarloFlow):
    """Importance sampling (vflow.py:215)."""

    _ALG = nat.VF_ALG_VEGAS
    _FUSED_F32_SAMPLER = True
    _GRAPH_ITERATIONS = True

    def __init__(self, n_dim, n_events, train=True, main_dimension=0, **kwargs):
        super().__init__(n_dim, n_events, **kwargs)
        self.train = train
        self.grid_bins = BINS_MAX + 1
        subdivision_np = np.linspace(0, 1, self.grid_bins)
        divisions_np = subdivision_np.repeat(n_dim).reshape(-1, n_dim).T
        self.divisions = torch.as_tensor(np.ascontiguousarray(divisions_np), dtype=torch.float64,
                                         device=self.device)
        self._main_dimension = main_dimension

    def _can_run_vectorial(self, expected_shape):
        if self._main_dimension >= expected_shape[-1]:
            raise ValueError(
                f"The main dimension index ({self._main_dimension}) is greater than the "
                f"dimensionality of the output ({expected_shape[-1]}). "
                "Remember that arrays in python are 0-indexed!")
        return self.__class__.__name__ == "VegasFlow"

    def _grid_ptr(self):
        return nat.ptr(self.divisions)

    def _train_now(self):
        return bool(self.train)

    # ---------------------------------------------------------------- grid control
    def freeze_grid(self):
        """Stops the grid from refining any more."""
        self.train = False
        self._recompile()

    def unfreeze_grid(self):
        """Enable the refining of the grid."""
        self.train = True
        self._recompile()

    def save_grid(self, file_name):
        """Save ``divisions`` as JSON (vflow.py:271-292)."""
        div_np = self.divisions.detach().cpu().numpy()
        int_name = getattr(self._integrand, "__name__", "") if self._integrand else ""
        json_dict = {
            "dimensions": self.n_dim,
            "ALPHA": ALPHA,
            "BINS": self.grid_bins,
            "integrand": int_name,
            "grid": div_np.tolist(),
        }
        with open(file_name, "w") as f:
            json.dump(json_dict, f, indent=True)

    def load_grid(self, file_name=None, numpy_grid=None):
        """Load ``divisions`` from a JSON file or an array (vflow.py:294-347)."""
        if file_name is not None and numpy_grid is not None:
            raise ValueError("Received both a numpy grid and a file_name to load the grid from."
                             "Ambiguous call to `load_grid`")
        if file_name:
            with open(file_name, "r") as f:
                json_dict = json.load(f)
            grid_dim = json_dict.get("dimensions")
            grid_bins = json_dict.get("BINS")
            if self._integrand:
                integrand_name = getattr(self._integrand, "__name__", "")
                integrand_grid = json_dict.get("integrand")
                if integrand_name != integrand_grid:
                    logger.warning(f"The grid was written for the integrand: {integrand_grid}"
                                   f"which is different from {integrand_name}")
            numpy_grid = np.array(json_dict["grid"])
        elif numpy_grid is not None:
            numpy_grid = np.asarray(numpy_grid)
            grid_dim = numpy_grid.shape[0]
            grid_bins = numpy_grid.shape[1]
        else:
            raise ValueError("load_grid was called but no grid was provided!")
        if grid_dim is not None and self.n_dim != grid_dim:
            raise ValueError(f"Received a {grid_dim}-dimensional grid while VegasFlow"
                             f"was instantiated with {self.n_dim} dimensions")
        if grid_bins is not None and self.grid_bins != grid_bins:
            raise ValueError(f"The received grid contains {grid_bins} bins while the"
                             f"current settings is of {self.grid_bins} bins")
        if numpy_grid.shape != tuple(self.divisions.shape):
            raise ValueError(f"grid of shape {numpy_grid.shape}, expected {tuple(self.divisions.shape)}")
        if file_name:
            logger.info(f" > SUCCESS: Loaded grid from {file_name}")
        self.divisions.copy_(torch.as_tensor(numpy_grid, dtype=torch.float64))

    def refine_grid(self, arr_res2):
        """Refine every dimension from the per-bin (w f)^2 sums (vflow.py:349-362)."""
        self._require_gpu()
        hist = torch.as_tensor(arr_res2, dtype=torch.float64, device=self.device).reshape(
            self.n_dim, BINS_MAX).contiguous()
        nat.call("vf_refine_grid", nat.ptr(self.divisions), nat.ptr(hist), self.n_dim, float(ALPHA),
                 nat.ptr(self._workspace()["flags"]) if self._rows else None, nat.stream_handle())

    # ---------------------------------------------------------------- sampling hooks
    def _digest_random_generation(self, rnds):
        """(x, w, ind) of the importance map applied to given uniforms
        (vflow.py:364-368 -> 93-126 -> 39-83); w is the map's Jacobian only."""
        self._require_gpu()
        u = torch.as_tensor(rnds, dtype=torch.float64, device=self.device).contiguous()
        n = u.shape[0]
        x = torch.empty((n, self.n_dim), dtype=self._rdtype, device=self.device)
        w = torch.empty(n, dtype=self._rdtype, device=self.device)
        ind = torch.empty((n, self.n_dim), dtype=torch.int32, device=self.device)
        nat.call("vf_sample", self._ALG, self._prec, nat.ptr(self.divisions), self.n_dim, int(n), 0,
                 1.0, None, None, 1.0, nat.ptr(u), self._seed, 0, nat.VF_INT_NONE, None, 0, 0, None, 1,
                 nat.ptr(ind), nat.ptr(x), nat.ptr(w), None, None, nat.stream_handle())
        return x, w, ind

    def _importance_sampling_array_filling(self, results2, indices):
        """(n_dim, 50) per-bin sums of ``results2`` (vflow.py:370-387)."""
        from .utils import consume_array_into_indices
        if not self.train:
            return []
        return torch.stack([consume_array_into_indices(results2, indices[:, j:j + 1], BINS_MAX)
                            for j in range(self.n_dim)])

    def _run_event(self, integrand, ncalls=None):
        """res, res2, arr_res2 of one chunk of ``ncalls`` events (vflow.py:389-430)."""
        if ncalls is None or int(ncalls) == self.n_events:
            return self.run_event()
        return self._event_sums(int(ncalls))

    def _iteration_content(self):
        """Sample, reduce, sigma, refine (vflow.py:432-442) -- two kernel launches."""
        self._fill_partials(train=self.train)
        return self._end_iteration(train=self.train)

    def _run_iteration(self):
        return self._iteration_content()


def vegas_wrapper(integrand, n_dim, n_iter, total_n_events, **kwargs):
    """Convenience wrapper (vflow.py:449-464)."""
    return wrapper(VegasFlow, integrand, n_dim, n_iter, total_n_events, **kwargs)


def vegas_sampler(*args, **kwargs):
    """Train a grid and return its ``generate_random_array`` (vflow.py:467-481)."""
    return sampler(VegasFlow, *args, **kwargs)
