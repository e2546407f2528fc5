// Calibration kernel for the issue-rate roofline of the fused sampler: eight
// independent fp32 FMA chains per thread keep every SM sub-partition issuing
// one warp instruction per clock.  Used by bench.py to measure the achievable
// warp-instruction rate at the clocks of the run.
#include "vegasflow_gb300.h"
#include "vf_internal.h"

#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(256) vf_issue_probe_kernel(float* out, int iters) {
  float a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = threadIdx.x * 1e-3f + j;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int r = 0; r < 16; ++r) {
#pragma unroll
      for (int j = 0; j < 8; ++j) a[j] = fmaf(a[j], 0.99999f, 1e-7f);
    }
  }
  float s = 0.0f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int vf_issue_probe(float* out, int blocks, int iters, long long* fma_per_thread, void* stream) {
  if (!out || blocks < 1 || iters < 1) return VF_ERR_ARG;
  vf_issue_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, iters);
  if (fma_per_thread) *fma_per_thread = 8LL * 16LL * iters;
  return cudaGetLastError() == cudaSuccess ? VF_OK : VF_ERR_LAUNCH;
}

namespace vf {
cudaError_t preload_probe_kernels() {
  cudaFuncAttributes attr;
  return cudaFuncGetAttributes(&attr, vf_issue_probe_kernel);
}
}  // namespace vf
