// An allocation-free VEGAS iteration for callers that cannot allocate device
// memory.
//
// Some callers of this library run where cudaMalloc is not available to them:
// plugins inside a host framework that owns all device memory through its own
// pool, code running inside a CUDA stream capture that must not allocate, or
// environments with a fixed memory budget.  The other entry points ask the
// caller for the block-partial scratch (`partials`); this one keeps that
// scratch in a fixed array inside the library instead, so the caller passes
// only its inputs and outputs.
//
// The scratch is a file-scope __device__ array of VF_STATIC_SCRATCH_BYTES
// (4 MiB of partial rows plus a small state area).  Every GPU that loads the
// library holds it until the process exits.  All calls share it and it keeps
// the previous call's contents: the state words that must start at zero are
// cleared by each call, and calls whose work overlaps on the GPU (two streams,
// two threads) race on it, so callers must order them.
#include <mutex>

#include <cuda_runtime.h>

#include "vegasflow_gb300.h"
#include "vf_internal.h"

#define VF_STATIC_ROW_DOUBLES (1 << 19)  // 4 MiB of block-partial rows
#define VF_STATIC_STATE_DOUBLES 16       // history (2), average (5), flags
#define VF_STATIC_SCRATCH_BYTES ((VF_STATIC_ROW_DOUBLES + VF_STATIC_STATE_DOUBLES) * 8)

static __device__ __align__(256) double vf_static_scratch[VF_STATIC_ROW_DOUBLES + VF_STATIC_STATE_DOUBLES];

namespace {

std::mutex g_static_mu;
constexpr int kMaxDevices = 128;
double* g_static_ptr[kMaxDevices] = {};

// Device address of the scratch on the current device (resolved once per device:
// in host code the array's name is not a device address).
int static_scratch(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return vf::set_error(VF_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return vf::set_error(VF_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, vf_static_scratch);
    if (e != cudaSuccess || !p)
      return vf::set_error(VF_ERR_CUDA, "cudaGetSymbolAddress(vf_static_scratch) failed");
    g_static_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_static_ptr[dev];
  return VF_OK;
}

}  // namespace

extern "C" int vf_vegas_iteration_static(int precision, double* grid, int n_dim, long long n_events,
                                         unsigned long long seed, unsigned int call_ctr, int integrand,
                                         const double* params, int train, double* res_sigma,
                                         void* stream) {
  if (!grid || !res_sigma) return vf::set_error(VF_ERR_ARG, "vf_vegas_iteration_static: NULL grid or output");
  if (n_dim < 1 || n_dim > VF_MAX_DIM)
    return vf::set_error(VF_ERR_UNSUPPORTED, "vf_vegas_iteration_static: n_dim must be 1..16");
  if (n_events < 2) return vf::set_error(VF_ERR_ARG, "vf_vegas_iteration_static: n_events must be >= 2");
  if (integrand < VF_INT_SYMGAUSS || integrand > VF_INT_SUM)
    return vf::set_error(VF_ERR_ARG, "vf_vegas_iteration_static: a built-in integrand id is required");
  const long long width = 2 + (long long)VF_BINS_MAX * n_dim;
  const long long max_rows = VF_STATIC_ROW_DOUBLES / width;
  if (max_rows < 1)
    return vf::set_error(VF_ERR_UNSUPPORTED, "vf_vegas_iteration_static: partial rows exceed the 4 MiB scratch");
  double* base = nullptr;
  int rc = static_scratch(&base);
  if (rc) return rc;
  int rows = 0;
  rc = vf_sample_rows(VF_ALG_VEGAS, precision, n_dim, integrand, train, &rows);
  if (rc) return rc;
  if (rows > max_rows) rows = (int)max_rows;  // the sampler is grid-stride: fewer rows is fine
  double* partials = base;
  double* state = base + VF_STATIC_ROW_DOUBLES;
  double* history = state;     // [res, sigma]
  double* avg = state + 2;     // running average (5 doubles), starts at zero
  int* flags = reinterpret_cast<int*>(state + 8);
  cudaError_t e = cudaMemsetAsync(state, 0, VF_STATIC_STATE_DOUBLES * sizeof(double), (cudaStream_t)stream);
  if (e != cudaSuccess) return vf::set_error(VF_ERR_CUDA, cudaGetErrorString(e));
  rc = vf_sample(VF_ALG_VEGAS, precision, grid, n_dim, n_events, 0, 1.0 / (double)n_events, nullptr,
                 nullptr, 1.0, nullptr, seed, call_ctr, integrand, params, train, 0, partials, rows,
                 nullptr, nullptr, nullptr, nullptr, flags, stream);
  if (rc) return rc;
  rc = vf_iteration_end(partials, rows, n_dim, 1, train, (double)n_events, 1.5, grid, nullptr, nullptr,
                        history, avg, 0, flags, stream);
  if (rc) return rc;
  e = cudaMemcpyAsync(res_sigma, history, 2 * sizeof(double), cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
  if (e != cudaSuccess) return vf::set_error(VF_ERR_CUDA, cudaGetErrorString(e));
  return VF_OK;
}
