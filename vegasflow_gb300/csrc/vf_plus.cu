// VEGAS+ entry points (vf_plus_*) and the ahead-of-time instantiations of the
// stratified sampler.
#include <cuda_runtime.h>

#include <cstdio>
#include <map>
#include <mutex>
#include <utility>

#include "vegasflow_gb300.h"
#include "vf_internal.h"
#include "vf_plus.cuh"
#include "vf_plus_f32.cuh"

namespace {

template <typename Real, int DMAX>
const void* pick(int integrand) {
  switch (integrand) {
    case VF_INT_NONE: return (const void*)vf::vf_plus_kernel<Real, DMAX, VF_INT_NONE>;
    case VF_INT_SYMGAUSS: return (const void*)vf::vf_plus_kernel<Real, DMAX, VF_INT_SYMGAUSS>;
    case VF_INT_GAUSS: return (const void*)vf::vf_plus_kernel<Real, DMAX, VF_INT_GAUSS>;
    case VF_INT_BREIT_WIGNER: return (const void*)vf::vf_plus_kernel<Real, DMAX, VF_INT_BREIT_WIGNER>;
    case VF_INT_PROD: return (const void*)vf::vf_plus_kernel<Real, DMAX, VF_INT_PROD>;
    case VF_INT_SUM: return (const void*)vf::vf_plus_kernel<Real, DMAX, VF_INT_SUM>;
    default: return nullptr;
  }
}

const void* plus_kernel(int precision, int n_dim, int integrand) {
  const int dmax = vf::dim_bucket(n_dim);
  if (precision == VF_PREC_F64) {
    if (dmax == 4) return pick<double, 4>(integrand);
    if (dmax == 8) return pick<double, 8>(integrand);
    return pick<double, 16>(integrand);
  }
  if (dmax == 4) return pick<float, 4>(integrand);
  if (dmax == 8) return pick<float, 8>(integrand);
  return pick<float, 16>(integrand);
}

int err(int code, const char* msg) { return vf::set_error(code, msg); }

int launched(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return err(VF_ERR_LAUNCH, buf);
  }
  return VF_OK;
}

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n;
}

// Raise a VEGAS+ sampler's dynamic shared-memory limit once per (device, kernel)
// and size (launches inside a stream capture then make no attribute calls).
int plus_prepare_smem(const void* k, int smem) {
  if (smem <= 48 * 1024) return VF_OK;
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, int> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(dev, k);
  const auto it = done.find(key);
  if (it != done.end() && it->second >= smem) return VF_OK;
  const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return err(VF_ERR_CUDA, cudaGetErrorString(e));
  done[key] = smem;
  return VF_OK;
}

// Resident blocks per SM of the VEGAS+ sampler that Philox iterations launch for
// (precision, n_dim) -- in fp32 the float32 kernel, in float64 the generic one --
// the smallest over the built-in integrands; computed once per configuration.
int plus_blocks_per_sm(int precision, int n_dim) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(precision, n_dim);
  const auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int best = 0;
  for (int integ = VF_INT_SYMGAUSS; integ <= VF_INT_SUM; ++integ) {
    const bool f32 = precision == VF_PREC_F32;
    const void* k = f32 ? vf::plus_f32_kernel(n_dim, integ) : plus_kernel(precision, n_dim, integ);
    const int smem = f32 ? vf::plus_f32_smem_bytes(n_dim, 1) : vf::plus_smem_bytes(8, n_dim, 1);
    int per_sm = 0;
    if (k && plus_prepare_smem(k, smem) == VF_OK &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, VF_THREADS, smem) == cudaSuccess &&
        per_sm > 0 && (best == 0 || per_sm < best))
      best = per_sm;
  }
  if (best == 0) best = 1;
  cache[key] = best;
  return best;
}

}  // namespace

extern "C" {

int vf_plus_rows(int precision, int n_dim, int n_hcubes, int* rows) {
  if (!rows || n_dim < 1 || n_dim > VF_MAX_DIM || n_hcubes < 1)
    return err(VF_ERR_ARG, "vf_plus_rows: bad arguments");
  if (precision != VF_PREC_F64 && precision != VF_PREC_F32) return err(VF_ERR_ARG, "vf_plus_rows: precision");
  const int sms = sm_count();
  if (sms <= 0) return err(VF_ERR_CUDA, "vf_plus_rows: no CUDA device");
  // one warp per hypercube, at most one wave of resident blocks: a second,
  // partial wave would hold the iteration for a whole hypercube's time
  int need = (n_hcubes + VF_THREADS / 32 - 1) / (VF_THREADS / 32);
  const int cap = plus_blocks_per_sm(precision, n_dim) * sms;
  *rows = need < cap ? need : cap;
  return VF_OK;
}

}  // extern "C"

namespace {

// vf_plus_sample with, optionally, the Philox call counter in device memory.
int plus_sample_impl(int precision, const double* grid, int n_dim, int n_strat, int n_hcubes, const int* n_ev,
                     const long long* ev_start, double xjac, const double* xmin, const double* xdelta,
                     double xdeltajac, const double* u_inj, unsigned long long seed, unsigned int call_ctr,
                     const unsigned int* call_dev, int integrand, const double* params, int train, double* ress,
                     double* ress2, double* partials, int rows, int* ind_out, void* x_out, void* w_out, int* flags,
                     void* stream) {
  if (precision != VF_PREC_F64 && precision != VF_PREC_F32) return err(VF_ERR_ARG, "vf_plus_sample: precision");
  if (n_dim < 1 || n_dim > VF_MAX_DIM) return err(VF_ERR_UNSUPPORTED, "vf_plus_sample: n_dim must be 1..16");
  if (!grid || !n_ev || !ev_start || n_strat < 1 || n_hcubes < 1 || rows < 1)
    return err(VF_ERR_ARG, "vf_plus_sample: NULL buffer or bad stratification");
  if ((xmin == nullptr) != (xdelta == nullptr)) return err(VF_ERR_ARG, "vf_plus_sample: xmin/xdelta");
  const bool jit = integrand >= VF_INT_JIT_BASE;
  if ((integrand < VF_INT_NONE || integrand > VF_INT_SUM) && !jit) return err(VF_ERR_ARG, "vf_plus_sample: integrand");
  if (integrand != VF_INT_NONE && (!ress || !ress2 || !partials))
    return err(VF_ERR_ARG, "vf_plus_sample: ress/ress2/partials required when evaluating");
  if ((integrand == VF_INT_SYMGAUSS || integrand == VF_INT_GAUSS || integrand == VF_INT_BREIT_WIGNER) && !params)
    return err(VF_ERR_ARG, "vf_plus_sample: integrand needs params");
  // fp32 with a built-in integrand and Philox uniforms: the float32 kernel
  const bool f32_tap = !jit && precision == VF_PREC_F32 && !u_inj && ind_out && !w_out &&
                       (integrand == VF_INT_SYMGAUSS || integrand == VF_INT_BREIT_WIGNER);
  const bool f32 = f32_tap || (precision == VF_PREC_F32 && integrand >= VF_INT_SYMGAUSS &&
                               integrand <= VF_INT_SUM && !u_inj && !ind_out && !x_out && !w_out);
  const void* k = jit       ? nullptr
                  : f32_tap ? vf::plus_f32_tap_kernel(n_dim, integrand)
                  : f32     ? vf::plus_f32_kernel(n_dim, integrand)
                            : plus_kernel(precision, n_dim, integrand);
  if (!k && !jit) return err(VF_ERR_UNSUPPORTED, "vf_plus_sample: no kernel");
  vf::PlusArgs a;
  a.grid = grid;
  a.n_ev = n_ev;
  a.ev_start = ev_start;
  a.xmin = xmin;
  a.xdelta = xdelta;
  a.u_inj = u_inj;
  a.params = params;
  a.ress = ress;
  a.ress2 = ress2;
  a.partials = partials;
  a.ind_out = ind_out;
  a.x_out = x_out;
  a.w_out = w_out;
  a.flags = flags;
  a.xjac = xjac;
  a.xdeltajac = xmin ? xdeltajac : 1.0;
  a.n_dim = n_dim;
  a.n_strat = n_strat;
  a.n_hcubes = n_hcubes;
  a.train = train ? 1 : 0;
  unsigned int k0 = (unsigned int)seed, k1 = (unsigned int)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    a.rk.k0[r] = k0;
    a.rk.k1[r] = k1;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  for (int q = 0; q < 8; ++q) a.ctr2[q] = (call_ctr << 4) | (unsigned int)q;
  a.ctr3 = call_ctr >> 28;
  a.call_dev = call_dev;
  if (jit) {
    const bool fast = precision == VF_PREC_F32 && !u_inj && !ind_out && !x_out && !w_out;
    const int rc = vf::jit_launch_plus(integrand, precision, n_dim, &a, rows, a.train, fast, stream);
    return rc ? rc : launched("vf_plus_sample (JIT)");
  }
  const int smem = f32 ? vf::plus_f32_smem_bytes(n_dim, a.train)
                       : vf::plus_smem_bytes(precision == VF_PREC_F64 ? 8 : 4, n_dim, a.train);
  const int rs = plus_prepare_smem(k, smem);
  if (rs != VF_OK) return rs;
  void* args[] = {&a};
  const cudaError_t e = cudaLaunchKernel(k, dim3(rows), dim3(VF_THREADS), args, smem, (cudaStream_t)stream);
  if (e != cudaSuccess) return err(VF_ERR_LAUNCH, cudaGetErrorString(e));
  return launched("vf_plus_sample");
}

// vf_plus_iteration_end with, optionally, the iteration index and the Philox
// call counter in device memory (read, then advanced).
int plus_end_impl(const double* ress, const double* ress2, int* n_ev, long long* ev_start, int n_hcubes, int adaptive,
                  int min_neval, double init_calls, const double* partials, int rows, int n_dim, int train,
                  double alpha, double beta, double* grid, double* hist_out, double* arr_var_out, double* history,
                  double* avg, int iter, int* iter_dev, unsigned int* call_dev, int hist_cap, int* flags,
                  void* stream) {
  if (!ress || !ress2 || !n_ev || !ev_start || !history || !avg || n_hcubes < 1 || iter < 0)
    return err(VF_ERR_ARG, "vf_plus_iteration_end: NULL buffer");
  if (n_dim < 1 || n_dim > VF_MAX_DIM) return err(VF_ERR_UNSUPPORTED, "vf_plus_iteration_end: n_dim");
  if ((train || hist_out) && (!partials || rows < 1)) return err(VF_ERR_ARG, "vf_plus_iteration_end: partials");
  if (train && !grid) return err(VF_ERR_ARG, "vf_plus_iteration_end: grid required when train");
  if (adaptive && min_neval < 1) return err(VF_ERR_ARG, "vf_plus_iteration_end: min_neval");
  if (n_hcubes > VF_PEND_CLUSTER * VF_PEND_THREADS * VF_PEND_MAXC)
    return err(VF_ERR_UNSUPPORTED, "vf_plus_iteration_end: more than 16384 hypercubes");
  if (train < 0 || train > 2) return err(VF_ERR_ARG, "vf_plus_iteration_end: train must be 0, 1 or 2");
  if (iter_dev && hist_cap < 1) return err(VF_ERR_ARG, "vf_plus_iteration_end: hist_cap");
  vf::PlusEndArgs a;
  a.ress = ress;
  a.ress2 = ress2;
  a.n_ev = n_ev;
  a.ev_start = ev_start;
  a.arr_var = arr_var_out;
  a.partials = partials;
  a.grid = grid;
  a.hist_out = hist_out;
  a.history = history;
  a.avg = avg;
  a.flags = flags;
  a.init_calls = init_calls;
  a.alpha = alpha;
  a.beta = beta;
  a.n_hcubes = n_hcubes;
  a.min_neval = min_neval;
  a.adaptive = adaptive ? 1 : 0;
  a.rows = rows;
  a.n_dim = n_dim;
  a.train = train;
  a.iter = iter;
  a.iter_dev = iter_dev;
  a.call_dev = call_dev;
  a.hist_cap = hist_cap;
  const int clusters = (a.train || hist_out) ? n_dim + 1 : 1;
  vf::vf_plus_iteration_end_kernel<<<clusters * VF_PEND_CLUSTER, VF_PEND_THREADS, 0, (cudaStream_t)stream>>>(a);
  return launched("vf_plus_iteration_end");
}

}  // namespace

extern "C" {

int vf_plus_sample(int precision, const double* grid, int n_dim, int n_strat, int n_hcubes,
                   const int* n_ev, const long long* ev_start, double xjac, const double* xmin,
                   const double* xdelta, double xdeltajac, const double* u_inj,
                   unsigned long long seed, unsigned int call_ctr, int integrand, const double* params,
                   int train, double* ress, double* ress2, double* partials, int rows, int* ind_out,
                   void* x_out, void* w_out, int* flags, void* stream) {
  return plus_sample_impl(precision, grid, n_dim, n_strat, n_hcubes, n_ev, ev_start, xjac, xmin, xdelta, xdeltajac,
                          u_inj, seed, call_ctr, nullptr, integrand, params, train, ress, ress2, partials, rows,
                          ind_out, x_out, w_out, flags, stream);
}

int vf_plus_reduce_events(int precision, const void* f, const void* w, const int* ind, const int* n_ev,
                          const long long* ev_start, int n_dim, int n_hcubes, int train, double* ress,
                          double* ress2, double* partials, int rows, void* stream) {
  if (!f || !w || !n_ev || !ev_start || !ress || !ress2 || !partials || rows < 1 || n_hcubes < 1)
    return err(VF_ERR_ARG, "vf_plus_reduce_events: NULL buffer");
  if (n_dim < 1 || n_dim > VF_MAX_DIM) return err(VF_ERR_UNSUPPORTED, "vf_plus_reduce_events: n_dim");
  if (train && !ind) return err(VF_ERR_ARG, "vf_plus_reduce_events: ind required when train");
  vf::PlusReduceArgs a;
  a.f = f;
  a.w = w;
  a.ind = ind;
  a.n_ev = n_ev;
  a.ev_start = ev_start;
  a.ress = ress;
  a.ress2 = ress2;
  a.partials = partials;
  a.n_dim = n_dim;
  a.n_hcubes = n_hcubes;
  a.train = train ? 1 : 0;
  const int smem = n_dim * VF_BINS * 8;
  if (precision == VF_PREC_F64)
    vf::vf_plus_reduce_kernel<double><<<rows, VF_THREADS, smem, (cudaStream_t)stream>>>(a);
  else if (precision == VF_PREC_F32)
    vf::vf_plus_reduce_kernel<float><<<rows, VF_THREADS, smem, (cudaStream_t)stream>>>(a);
  else
    return err(VF_ERR_ARG, "vf_plus_reduce_events: precision");
  return launched("vf_plus_reduce_events");
}

int vf_plus_iteration_end(const double* ress, const double* ress2, int* n_ev, long long* ev_start,
                          int n_hcubes, int adaptive, int min_neval, double init_calls,
                          const double* partials, int rows, int n_dim, int train, double alpha,
                          double beta, double* grid, double* hist_out, double* arr_var_out,
                          double* history, double* avg, int iter, int* flags, void* stream) {
  return plus_end_impl(ress, ress2, n_ev, ev_start, n_hcubes, adaptive, min_neval, init_calls, partials, rows, n_dim,
                       train, alpha, beta, grid, hist_out, arr_var_out, history, avg, iter, nullptr, nullptr, 0, flags,
                       stream);
}

int vf_plus_iteration_dev(int precision, double* grid, int n_dim, int n_strat, int n_hcubes, int* n_ev,
                          long long* ev_start, double xjac, const double* xmin, const double* xdelta,
                          double xdeltajac, unsigned long long seed, unsigned int* call_dev, int* iter_dev,
                          int integrand, const double* params, int train, int adaptive, int min_neval,
                          double init_calls, double alpha, double beta, double* ress, double* ress2,
                          double* partials, int rows, double* history, int hist_cap, double* avg, int* flags,
                          void* stream) {
  if (!call_dev || !iter_dev) return err(VF_ERR_ARG, "vf_plus_iteration_dev: call_dev and iter_dev are required");
  if (integrand == VF_INT_NONE) return err(VF_ERR_ARG, "vf_plus_iteration_dev: needs an integrand");
  int rc = plus_sample_impl(precision, grid, n_dim, n_strat, n_hcubes, n_ev, ev_start, xjac, xmin, xdelta, xdeltajac,
                            nullptr, seed, 0, call_dev, integrand, params, train, ress, ress2, partials, rows, nullptr,
                            nullptr, nullptr, flags, stream);
  if (rc) return rc;
  const int tr = train ? (precision == VF_PREC_F32 ? 2 : 1) : 0;
  return plus_end_impl(ress, ress2, n_ev, ev_start, n_hcubes, adaptive, min_neval, init_calls, partials, rows, n_dim,
                       tr, alpha, beta, grid, nullptr, nullptr, history, avg, 0, iter_dev, call_dev, hist_cap, flags,
                       stream);
}

}  // extern "C"

namespace vf {
cudaError_t preload_plus_kernels() {
  cudaFuncAttributes attr;
  for (int prec = 0; prec < 2; ++prec)
    for (int dmax : {4, 8, 16})
      for (int integ = VF_INT_NONE; integ <= VF_INT_SUM; ++integ) {
        const void* k = ::plus_kernel(prec ? VF_PREC_F32 : VF_PREC_F64, dmax, integ);
        if (k) {
          const cudaError_t e = cudaFuncGetAttributes(&attr, k);
          if (e != cudaSuccess) return e;
        }
      }
  for (int d = 1; d <= VF_MAX_DIM; ++d)
    for (int integ = VF_INT_SYMGAUSS; integ <= VF_INT_SUM; ++integ) {
      const cudaError_t e = cudaFuncGetAttributes(&attr, plus_f32_kernel(d, integ));
      if (e != cudaSuccess) return e;
    }
  cudaError_t e = cudaFuncGetAttributes(&attr, vf_plus_reduce_kernel<double>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&attr, vf_plus_reduce_kernel<float>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&attr, vf_plus_iteration_end_kernel);
  return e;
}
}  // namespace vf
