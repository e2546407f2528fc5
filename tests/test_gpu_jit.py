"""CUDA-source integrands compiled by NVRTC into the sampler."""

import math

import numpy as np
import pytest
import torch

from vegasflow_gb300 import PlainFlow, VegasFlow, VegasFlowPlus, integrands

pytestmark = pytest.mark.gpu

CAMEL_SRC = """
__device__ vf_real camel(const vf_real* x, int n_dim, vf_real weight, const double* params) {
  vf_real s1 = 0, s2 = 0;
  for (int d = 0; d < n_dim; ++d) {
    const vf_real t1 = (x[d] - (vf_real)params[0]) / (vf_real)params[2];
    const vf_real t2 = (x[d] - (vf_real)params[1]) / (vf_real)params[2];
    s1 += t1 * t1;
    s2 += t2 * t2;
  }
  return exp(-s1) + exp(-s2);
}
"""
P = [0.3, 0.7, 0.1]


def camel_torch(x, weight=None):
    return (torch.exp(-torch.sum(((x - P[0]) / P[2]) ** 2, dim=1))
            + torch.exp(-torch.sum(((x - P[1]) / P[2]) ** 2, dim=1)))


def camel_exact(d):
    one = lambda m: P[2] * math.sqrt(math.pi) / 2 * (math.erf((1 - m) / P[2]) + math.erf(m / P[2]))  # noqa: E731
    return one(P[0]) ** d + one(P[1]) ** d


@pytest.mark.parametrize("cls,precision", [(VegasFlow, "fp32"), (VegasFlow, "fp64"), (PlainFlow, "fp32"),
                                           (VegasFlowPlus, "fp32"), (VegasFlowPlus, "fp64")])
def test_camel_against_exact(cls, precision):
    d = 4
    inst = cls(d, 1_000_000, verbose=False, precision=precision, seed=3)
    inst.compile(integrands.cuda_integrand(CAMEL_SRC, "camel", params=P))
    res, sigma = inst.run_integration(5)
    assert abs(res - camel_exact(d)) < 5 * sigma, (res, sigma, camel_exact(d))


def test_fp64_jit_equals_torch_callable():
    """Same Philox stream, same points: the device function and the torch
    callable give the same iterations to rounding."""
    out = []
    for f in (integrands.cuda_integrand(CAMEL_SRC, "camel", params=P), camel_torch):
        inst = VegasFlow(3, 200_000, verbose=False, precision="fp64", seed=8)
        inst.compile(f)
        out.append(np.array([[float(v) for v in inst._run_iteration()] for _ in range(3)]))
    np.testing.assert_allclose(out[0], out[1], rtol=1e-10)


def test_weight_argument_is_the_full_weight():
    """The integrand's `weight` is the event's full weight (map Jacobian x 1/N),
    as the reference passes it (monte_carlo.py:583-591)."""
    src = "__device__ vf_real wgt(const vf_real* x, int n_dim, vf_real weight, const double* p) { return weight; }"
    out = []
    for f in (integrands.cuda_integrand(src, "wgt"), lambda x, weight=None: weight):
        inst = VegasFlow(2, 50_000, verbose=False, precision="fp64", seed=4)
        inst.compile(f)
        out.append(float(inst._run_iteration()[0]))
    np.testing.assert_allclose(out[0], out[1], rtol=1e-12)


def test_jit_error_is_reported():
    bad = integrands.cuda_integrand("__device__ vf_real bad(const vf_real* x) { return y; }", "bad")
    inst = VegasFlow(2, 1000, verbose=False)
    with pytest.raises(RuntimeError, match="NVRTC"):
        inst.compile(bad)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_plus_cuda_integrand_matches_builtin(precision):
    """The same Gaussian as a CUDA-source integrand and as the built-in one in
    VEGAS+ (adaptive): same estimate within the two sigmas."""
    src = """
__device__ vf_real g(const vf_real* x, int n_dim, vf_real weight, const double* p) {
  vf_real s = 0;
  for (int d = 0; d < n_dim; ++d) { vf_real t = (x[d] - (vf_real)0.5) / (vf_real)p[0]; s += t * t; }
  return (vf_real)p[1] * exp(-s);
}
"""
    a = 0.2
    pref = (1.0 / a / math.sqrt(math.pi)) ** 3
    out = []
    for f in (integrands.cuda_integrand(src, "g", params=[a, pref]), integrands.symgauss(a)):
        inst = VegasFlowPlus(3, 400_000, adaptive=True, verbose=False, precision=precision, seed=12)
        inst.compile(f)
        out.append(inst.run_integration(4))
    (r1, s1), (r2, s2) = out
    assert abs(r1 - r2) < 5 * math.hypot(s1, s2), out
    assert abs(r1 - math.erf(0.5 / a) ** 3) < 5 * s1
