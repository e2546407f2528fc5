"""NVRTC compiles every sampler a CUDA-source integrand can be built into (no
GPU needed: ``vf_jit_check`` compiles without loading), so a header that nvcc
accepts but NVRTC rejects fails here on the CPU."""

import ctypes

import pytest

from vegasflow_gb300 import _native as nat

SRC = (b"__device__ vf_real camel(const vf_real* x, int n, vf_real w, const double* p) {"
       b" vf_real s = 0; for (int i = 0; i < n; ++i) s += x[i] * x[i]; return exp(-s); }")


@pytest.mark.parametrize("alg,precision,n_dim", [
    (nat.VF_ALG_VEGAS, nat.VF_PREC_F32, 8),   # fp32 Philox and injected-uniform kernels
    (nat.VF_ALG_VEGAS, nat.VF_PREC_F64, 3),   # generic sampler
    (nat.VF_ALG_PLAIN, nat.VF_PREC_F32, 2),
    (nat.VF_ALG_PLUS, nat.VF_PREC_F32, 6),    # VEGAS+ float64-map and float32 samplers
    (nat.VF_ALG_BATCH, nat.VF_PREC_F32, 16),  # batched sampler, dimension class 16
])
def test_nvrtc_builds_the_sampler(alg, precision, n_dim):
    log = ctypes.create_string_buffer(16384)
    rc = nat.load().vf_jit_check(SRC, b"camel", alg, precision, n_dim, log, len(log))
    assert rc == nat.VF_OK, log.value.decode(errors="replace")
