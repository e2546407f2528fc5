"""Integrands that run inside the fused sampler kernel.

``compile()`` accepts either a torch callable (evaluated on the sampler's x in
HBM, then reduced by a kernel) or one of the objects below, which the sampler
evaluates per event in registers: no x/w/f round trip through HBM.  Built-ins
cover the workloads of the configurations (normalised symmetric Gaussian,
per-dimension Gaussian, Breit-Wigner times linear factors) and two simple
test integrands; ``cuda_integrand`` JIT-compiles a user's CUDA device function
into the same sampler.

Each built-in object is also callable on torch tensors with the reference's
integrand signature ``f(xarr, weight=None, n_dim=None)`` (same formula,
evaluated by torch), which the tests use as the plain float64 comparison.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from . import _native as nat


class DeviceIntegrand:
    """An integrand evaluated inside the sampler kernel.

    ``integrand_id`` is a ``VF_INT_*`` id; ``params(n_dim)`` returns its float64
    parameter array (copied to the device at compile time)."""

    def __init__(self, integrand_id, name, params=None, torch_fn=None, n_dim=None):
        self.integrand_id = int(integrand_id)
        self.__name__ = name
        self._params = params
        self._torch_fn = torch_fn
        self.n_dim = n_dim

    def params(self, n_dim):
        if self._params is None:
            return np.zeros(1, dtype=np.float64)
        return np.asarray(self._params(n_dim), dtype=np.float64)

    def check_dims(self, n_dim):
        if self.n_dim is not None and self.n_dim != n_dim:
            raise ValueError(f"{self.__name__} was built for {self.n_dim} dimensions, not {n_dim}")

    def __call__(self, xarr, weight=None, n_dim=None, **kwargs):
        if self._torch_fn is None:
            raise NotImplementedError(f"{self.__name__} has no torch form")
        return self._torch_fn(xarr)

    def __repr__(self):
        return f"DeviceIntegrand({self.__name__})"


def symgauss(a=0.1):
    """prod_d exp(-(x_d - 1/2)^2 / a^2) / (a sqrt(pi)): the normalised Gaussian of
    the reference tests and examples (test_algs.py:27-36, simgauss_tf.py:22-32)."""

    def params(n_dim):
        return [a, (1.0 / a / math.sqrt(math.pi)) ** n_dim]

    def fn(x):
        n_dim = x.shape[-1]
        pref = (1.0 / a / math.sqrt(math.pi)) ** n_dim
        coef = torch.sum(((x - 0.5) / a) ** 2, dim=1)
        return pref * torch.exp(-coef)

    return DeviceIntegrand(nat.VF_INT_SYMGAUSS, "symgauss", params, fn)


def gauss(mu, a):
    """prod_d exp(-(x_d - mu_d)^2 / a_d^2), unnormalised (the batched workload)."""
    mu = np.asarray(mu, dtype=np.float64)
    a = np.asarray(a, dtype=np.float64)
    if mu.shape != a.shape or mu.ndim != 1:
        raise ValueError("mu and a must be 1-d arrays of the same length")

    def params(n_dim):
        return np.concatenate([mu, a])

    def fn(x):
        m = torch.as_tensor(mu, dtype=x.dtype, device=x.device)
        s = torch.as_tensor(a, dtype=x.dtype, device=x.device)
        return torch.exp(-torch.sum(((x - m) / s) ** 2, dim=1))

    return DeviceIntegrand(nat.VF_INT_GAUSS, "gauss", params, fn, n_dim=mu.size)


def gauss_exact(mu, a):
    out = 1.0
    for m, s in zip(mu, a):
        out *= s * math.sqrt(math.pi) / 2.0 * (math.erf((1.0 - m) / s) + math.erf(m / s))
    return out


def breit_wigner(coeffs, mass=91.19, width=2.50):
    """20000 / ((s - M^2)^2 + M^2 G^2) * prod_{d>=2}(1 + c_d x_d) with s = 2500 + 20000 x_1
    (s mapped linearly onto [50^2, 150^2], Jacobian included)."""
    coeffs = np.asarray(coeffs, dtype=np.float64)

    def params(n_dim):
        if coeffs.size < n_dim - 1:
            raise ValueError(f"breit_wigner needs {n_dim - 1} coefficients, got {coeffs.size}")
        return np.concatenate([[mass, width], coeffs[: n_dim - 1]])

    def fn(x):
        s = 2500.0 + 20000.0 * x[:, 0]
        m2 = mass * mass
        f = 20000.0 / ((s - m2) ** 2 + m2 * width * width)
        for d in range(1, x.shape[1]):
            f = f * (1.0 + float(coeffs[d - 1]) * x[:, d])
        return f

    return DeviceIntegrand(nat.VF_INT_BREIT_WIGNER, "breit_wigner", params, fn)


def breit_wigner_exact(n_dim, coeffs, mass=91.19, width=2.50):
    mg = mass * width
    m2 = mass * mass
    val = (math.atan((22500.0 - m2) / mg) - math.atan((2500.0 - m2) / mg)) / mg
    for d in range(1, n_dim):
        val *= 1.0 + coeffs[d - 1] / 2.0
    return val


def prod():
    """prod_d x_d (test_misc.py:24-26 ``_simple_integrand``)."""
    return DeviceIntegrand(nat.VF_INT_PROD, "prod", None, lambda x: torch.prod(x, dim=1))


def sum_():
    """sum_d x_d (the examples/cuda custom-op integrand)."""
    return DeviceIntegrand(nat.VF_INT_SUM, "sum", None, lambda x: torch.sum(x, dim=1))


class CudaIntegrand(DeviceIntegrand):
    """A user integrand written as a CUDA device function, compiled by NVRTC into
    the sampler (one specialised kernel per algorithm, precision and dimension
    count, compiled on first use and cached).

    ``source`` defines ``__device__ vf_real NAME(const vf_real* x, int n_dim,
    vf_real weight, const double* params)`` where ``vf_real`` is ``double`` or
    ``float`` following the integrator's precision; ``params`` (optional floats)
    reach the function as a device array.  ``torch_fn`` optionally gives the same
    integrand on torch tensors (for checks)."""

    def __init__(self, source, name, params=None, torch_fn=None, n_dim=None):
        super().__init__(-1, name, None, torch_fn, n_dim)
        self.source = source
        self._user_params = None if params is None else np.asarray(params, dtype=np.float64)
        self._ids = {}

    def params(self, n_dim):
        return self._user_params if self._user_params is not None else np.zeros(1)

    def compile_for(self, alg, precision, n_dim):
        """The integrand id of the kernel for (alg, precision, n_dim), compiling it if needed."""
        import ctypes

        key = (alg, precision, n_dim)
        if key not in self._ids:
            out = ctypes.c_int(0)
            nat.check(nat.load().vf_jit_integrand(self.source.encode(), self.__name__.encode(), alg, precision,
                                                  n_dim, ctypes.byref(out)))
            self._ids[key] = out.value
        return self._ids[key]

    def check(self, alg=0, precision=1, n_dim=4):
        """Compile without a GPU; returns (ok, NVRTC log)."""
        import ctypes

        buf = ctypes.create_string_buffer(1 << 16)
        rc = nat.load().vf_jit_check(self.source.encode(), self.__name__.encode(), alg, precision, n_dim, buf,
                                     len(buf))
        return rc == nat.VF_OK, buf.value.decode(errors="replace")


def cuda_integrand(source, name, params=None, torch_fn=None, n_dim=None):
    """Build a ``CudaIntegrand`` (see its docstring)."""
    return CudaIntegrand(source, name, params, torch_fn, n_dim)
