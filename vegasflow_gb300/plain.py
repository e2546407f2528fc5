"""PlainFlow: plain Monte Carlo (vegasflow plain.py:11-53)."""

from __future__ import annotations

from . import _native as nat
from .monte_carlo import MonteCarloFlow, sampler, wrapper


class PlainFlow(MonteCarloFlow):
    """Simple Monte Carlo integrator (plain.py:11)."""

    _CAN_RUN_VECTORIAL = True
    _ALG = nat.VF_ALG_PLAIN
    _GRAPH_ITERATIONS = True

    def _run_event(self, integrand, ncalls=None):
        """res, res2 of one chunk of ``ncalls`` events (plain.py:18-35)."""
        if ncalls is None or int(ncalls) == self.n_events:
            return self.run_event()
        return self._event_sums(int(ncalls))

    def _run_iteration(self):
        """plain.py:37-43: sigma from (res2 * N - res^2) / (N - 1)."""
        self._fill_partials(train=False)
        return self._end_iteration(train=False)


def plain_wrapper(*args, **kwargs):
    """Wrapper around PlainFlow (plain.py:46-48)."""
    return wrapper(PlainFlow, *args, **kwargs)


def plain_sampler(*args, **kwargs):
    """Wrapper sampler around PlainFlow (plain.py:51-53)."""
    return sampler(PlainFlow, *args, **kwargs)
