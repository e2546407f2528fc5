// Calibration kernel for the issue-rate roofline of the fused sampler: eight
// independent fp32 FMA chains per thread keep every SM sub-partition issuing
// one warp instruction per clock.  Used by bench.py to measure the achievable
// warp-instruction rate at the clocks of the run.
#include "vegasflow_gb300.h"
#include "vf_internal.h"
#include "vf_vegas_f32.cuh"

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

namespace {

// The same for the 64-bit integer multiply that Philox4x32-10 and the bin map
// issue (the FMA-heavy pipe): eight independent chains per thread of the
// Philox round's shape -- (hi, lo) = a * M, a' = hi ^ lo ^ k -- one wide
// multiply and one three-input XOR (the ALU pipe) per step, so the wide
// multiplies bound the chain's rate.
__global__ void __launch_bounds__(256) vf_widemul_probe_kernel(unsigned* out, int iters) {
  unsigned a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = threadIdx.x * 2654435761u + (unsigned)j;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int r = 0; r < 16; ++r) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const unsigned long long p = (unsigned long long)a[j] * 0xD2511F53ull;
        a[j] = (unsigned)(p >> 32) ^ (unsigned)p ^ 0x9E3779B9u;
      }
    }
  }
  unsigned s = 0u;
#pragma unroll
  for (int j = 0; j < 8; ++j) s ^= a[j];
  if (s == 0x12345678u) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int vf_widemul_probe(unsigned* out, int blocks, int iters, long long* mul_per_thread, void* stream) {
  if (!out || blocks < 1 || iters < 1) return VF_ERR_ARG;
  vf_widemul_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, iters);
  if (mul_per_thread) *mul_per_thread = 8LL * 16LL * iters;
  return cudaGetLastError() == cudaSuccess ? VF_OK : VF_ERR_LAUNCH;
}

namespace {

// The bounded wait of the TMA path, on a barrier that nothing completes: every
// thread gives up after `polls` polls and the block reports it.
__global__ void __launch_bounds__(64) vf_wait_selftest_kernel(int polls, int* flag) {
  __shared__ alignas(8) unsigned long long bar;
  const unsigned b = (unsigned)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(b), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool ok = vf::mbar_wait_bounded(b, 0u, polls);
  if (!__syncthreads_and(ok) && threadIdx.x == 0) atomicOr(flag, VF_FLAG_TIMEOUT);
}

}  // namespace

extern "C" int vf_wait_selftest(int polls, int* flag, void* stream) {
  if (!flag || polls < 1 || polls > (1 << 20)) return VF_ERR_ARG;
  vf_wait_selftest_kernel<<<1, 64, 0, (cudaStream_t)stream>>>(polls, flag);
  return cudaGetLastError() == cudaSuccess ? VF_OK : VF_ERR_LAUNCH;
}

namespace vf {
cudaError_t preload_probe_kernels() {
  cudaFuncAttributes attr;
  cudaError_t e = cudaFuncGetAttributes(&attr, vf_issue_probe_kernel);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&attr, vf_widemul_probe_kernel);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&attr, vf_wait_selftest_kernel);
  return e;
}
}  // namespace vf
