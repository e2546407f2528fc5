"""CPU oracle for the VEGAS hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy float64, what N3PDF/vegasflow computes on its
VEGAS sample -> map -> evaluate -> reduce -> refine path.  It exists to check
the CUDA implementation in ``vegasflow_gb300``; it is never the thing measured
or shipped.  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline / reference arm may import it.

Parity is pinned: ``tests/golden/make_golden.py`` runs the reference's own
Python modules (``src/vegasflow/*.py``) on a NumPy-backed stand-in for the
TensorFlow calls they make, with injected uniforms, and commits the outputs as
fixtures; ``tests/test_oracle_golden.py`` checks this oracle against them.
"""

from .vegas_oracle import *  # noqa: F401,F403
