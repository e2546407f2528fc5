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
#include <cuda.h>

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
// per device: the scratch's device address and the id of the context it was
// resolved in (a device reset makes a new context, where the array may sit
// elsewhere; the id, unique per context in the process, tells them apart)
double* g_static_ptr[kMaxDevices] = {};
unsigned long long g_static_ctx[kMaxDevices] = {};

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

template <typename Fn>
Fn driver_fn(const char* name) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    p = nullptr;
  return reinterpret_cast<Fn>(p);
}

// Id of the current context (0 when it cannot be had: then the address is
// resolved once per device, as without the id).
unsigned long long current_context_id() {
  static const PfnCtxGetCurrent get_current = driver_fn<PfnCtxGetCurrent>("cuCtxGetCurrent");
  static const PfnCtxGetId get_id = driver_fn<PfnCtxGetId>("cuCtxGetId");
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of the scratch on the current device.  In host code the
// array's name is a host-side stand-in, not a device address: it is resolved
// with cudaGetSymbolAddress once per device and context, with that device
// current (the first call on a device, which must come before any stream capture).
int static_scratch(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return vf::set_error(VF_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return vf::set_error(VF_ERR_UNSUPPORTED, "device index out of range");
  // id 0: no context is current yet (the lookup below makes the primary context
  // current, and the id is read after it) or the id cannot be read at all (then
  // every call resolves the address)
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_ptr[dev] || ctx == 0 || g_static_ctx[dev] != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, vf_static_scratch);
    if (e != cudaSuccess || !p)
      return vf::set_error(VF_ERR_CUDA, "cudaGetSymbolAddress(vf_static_scratch) failed");
    g_static_ptr[dev] = static_cast<double*>(p);
    g_static_ctx[dev] = current_context_id();
  }
  *out = g_static_ptr[dev];
  return VF_OK;
}

}  // namespace

extern "C" int vf_vegas_iteration_static(int precision, double* grid, int n_dim, long long n_events,
                                         unsigned long long seed, unsigned int call_ctr, int integrand,
                                         const double* params, int train, double* res_sigma, int* flags_out,
                                         void* stream) {
  if (!grid || !res_sigma) return vf::set_error(VF_ERR_ARG, "vf_vegas_iteration_static: NULL grid or output");
  if (precision != VF_PREC_F64 && precision != VF_PREC_F32)
    return vf::set_error(VF_ERR_ARG, "vf_vegas_iteration_static: precision must be VF_PREC_F64 or VF_PREC_F32");
  if (n_dim < 1 || n_dim > VF_MAX_DIM)
    return vf::set_error(VF_ERR_UNSUPPORTED, "vf_vegas_iteration_static: n_dim must be 1..16");
  if (n_events < 2) return vf::set_error(VF_ERR_ARG, "vf_vegas_iteration_static: n_events must be >= 2");
  if (integrand < VF_INT_SYMGAUSS || integrand > VF_INT_SUM)
    return vf::set_error(VF_ERR_ARG, "vf_vegas_iteration_static: a built-in integrand id is required");
  if (train < 0 || train > 2)
    return vf::set_error(VF_ERR_ARG, "vf_vegas_iteration_static: train must be 0, 1 or 2");
  const long long width = 2 + (long long)VF_BINS_MAX * n_dim;
  const long long max_rows = VF_STATIC_ROW_DOUBLES / width;
  if (max_rows < 1)
    return vf::set_error(VF_ERR_UNSUPPORTED, "vf_vegas_iteration_static: partial rows exceed the 4 MiB scratch");
  double* base = nullptr;
  int rc = static_scratch(&base);
  if (rc) return rc;
  const int fill = train != 0;  // the sampler fills the histogram; train picks the refinement
  int rows = 0;
  rc = vf_sample_rows(VF_ALG_VEGAS, precision, n_dim, integrand, fill, &rows);
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
                 nullptr, 1.0, nullptr, seed, call_ctr, integrand, params, fill, 0, partials, rows,
                 nullptr, nullptr, nullptr, nullptr, flags, stream);
  if (rc) return rc;
  rc = vf_iteration_end(partials, rows, n_dim, 1, train, (double)n_events, 1.5, grid, nullptr, nullptr,
                        history, avg, 0, flags, stream);
  if (rc) return rc;
  e = cudaMemcpyAsync(res_sigma, history, 2 * sizeof(double), cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
  if (e != cudaSuccess) return vf::set_error(VF_ERR_CUDA, cudaGetErrorString(e));
  if (flags_out) {
    e = cudaMemcpyAsync(flags_out, flags, sizeof(int), cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
    if (e != cudaSuccess) return vf::set_error(VF_ERR_CUDA, cudaGetErrorString(e));
  }
  return VF_OK;
}
