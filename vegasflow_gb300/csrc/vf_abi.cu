// The extern "C" entry points of libvegasgb.so (declared in
// include/vegasflow_gb300.h): argument checks, kernel selection, launch.
#include <cuda.h>

#include <atomic>
#include <cstdarg>
#include <map>
#include <tuple>
#include <mutex>
#include <cstdio>
#include <cstring>

#include "vegasflow_gb300.h"
#include "vf_internal.h"
#include "vf_iter.cuh"
#include "vf_sample.cuh"
#include "vf_map_f32.cuh"
#include "vf_vegas_f32.cuh"

namespace {

// Tunables (vf_tune_set): the histogram layout of the fp32 VEGAS sampler (0 =
// joint pair tables, the only layout)
std::atomic<int> g_f32_hist_copies{0};
// block size of the fp32 VEGAS Philox sampler (1024 | 512)
std::atomic<int> g_f32_threads{1024};
// persistent blocks per SM of the fp32 VEGAS sampler (0 = as many as fit): with
// the block size it sets the events each thread processes
std::atomic<int> g_f32_blocks_per_sm{0};

thread_local char g_err[1024] = "";

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int check_launch(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(VF_ERR_LAUNCH, "%s: %s", what, cudaGetErrorString(e));
  return VF_OK;
}

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  return n;
}

bool builtin_integrand(int id) { return id >= VF_INT_NONE && id <= VF_INT_SUM; }

// Per-warp histogram copies for fp32 (fewer same-address collisions), one block
// copy for float64 (shared float64 atomics, smem budget).
int hist_copies_for(int precision) { return precision == VF_PREC_F32 ? VF_THREADS / 32 : 1; }

const void* sample_kernel(int precision, int n_dim, int integrand) {
  const int dmax = vf::dim_bucket(n_dim);
  return precision == VF_PREC_F64 ? vf::sample_kernel_f64(dmax, integrand)
                                  : vf::sample_kernel_f32(dmax, integrand);
}

bool evaluating_builtin(int id) { return id >= VF_INT_SYMGAUSS && id <= VF_INT_SUM; }

// The specialised fp32 VEGAS kernel serves evaluating launches without taps.
bool use_vegas_f32(int alg, int precision, int integrand, bool taps) {
  return precision == VF_PREC_F32 && alg == VF_ALG_VEGAS && evaluating_builtin(integrand) && !taps;
}

// cuTensorMapEncodeTiled, resolved through the runtime (the library does not
// link the driver library).
typedef CUresult (*PfnTensorMapEncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                            const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                            CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                            CUtensorMapFloatOOBfill);

PfnTensorMapEncodeTiled tensor_map_encoder() {
  static PfnTensorMapEncodeTiled fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PfnTensorMapEncodeTiled>(p);
  }();
  return fn;
}

// The tensor map of injected uniforms [n][D] float64 with a box of `threads`
// rows, for D in {4, 8, 16} (rows of 32/64/128 bytes, swizzled by as many);
// returns the swizzle code (1|2|3) or 0 where the plain-load path applies.
int encode_uniform_tiles(vf::SampleArgs& a, const double* u, long long n, int D, int threads) {
  static_assert(sizeof(CUtensorMap) == sizeof(a.tmap), "tensor map size");
  const int code = D == 4 ? 1 : D == 8 ? 2 : D == 16 ? 3 : 0;
  if (!code || !u || (reinterpret_cast<size_t>(u) & 15) != 0 || n < 1 || n > (1ll << 31) - 1024) return 0;
  const PfnTensorMapEncodeTiled enc = tensor_map_encoder();
  if (!enc) return 0;
  const cuuint64_t dims[2] = {(cuuint64_t)D, (cuuint64_t)n};
  const cuuint64_t strides[1] = {(cuuint64_t)D * 8};
  const cuuint32_t box[2] = {(cuuint32_t)D, (cuuint32_t)threads};
  const cuuint32_t elem[2] = {1, 1};
  const CUtensorMapSwizzle swz = code == 1   ? CU_TENSOR_MAP_SWIZZLE_32B
                                 : code == 2 ? CU_TENSOR_MAP_SWIZZLE_64B
                                             : CU_TENSOR_MAP_SWIZZLE_128B;
  CUtensorMap* tm = reinterpret_cast<CUtensorMap*>(a.tmap);
  if (enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(u), dims, strides, box, elem,
          CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return 0;
  return code;
}

void fill_philox(vf::SampleArgs& a, unsigned long long seed, unsigned int call) {
  unsigned int k0 = (unsigned int)seed, k1 = (unsigned int)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    a.rk.k0[r] = k0;
    a.rk.k1[r] = k1;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  for (int q = 0; q < 8; ++q) a.ctr2[q] = (call << 4) | (unsigned int)q;
  a.ctr3 = call >> 28;
}

// Raise a kernel's dynamic shared-memory limit once per (device, kernel, size):
// later launches (and launches inside a stream capture) make no attribute call.
int prepare_smem(const void* kernel, int smem) {
  if (smem <= 48 * 1024) return VF_OK;
  int dev = 0;
  cudaGetDevice(&dev);
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, int> done;
  std::lock_guard<std::mutex> lock(mu);
  int& have = done[{dev, kernel}];
  if (have >= smem) return VF_OK;
  const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return fail(VF_ERR_CUDA, "cudaFuncSetAttribute(smem=%d): %s", smem, cudaGetErrorString(e));
  have = smem;
  return VF_OK;
}

// Blocks of `kernel` resident on the device at once (SMs x blocks per SM),
// cached per (device, kernel, block size, shared memory): launches make no
// occupancy query after the first.  0 on error.
int resident_blocks(const void* kernel, int threads, int smem) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  static std::mutex mu;
  static std::map<std::tuple<int, const void*, int, int>, int> cache;
  const auto key = std::make_tuple(dev, kernel, threads, smem);
  {
    std::lock_guard<std::mutex> lock(mu);
    const auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
    return 0;
  const int fit = per_sm * sm_count();
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = fit;
  return fit;
}

}  // namespace

namespace vf {
// Sets the calling thread's vf_last_error_string() for entry points defined in
// other translation units.
int set_error(int code, const char* message) { return fail(code, "%s", message); }
}  // namespace vf

extern "C" {

int vf_version(void) { return 1; }

int vf_tune_set(int key, int value) {
  if (key == VF_TUNE_F32_THREADS) {
    if (value != 512 && value != 1024) return fail(VF_ERR_ARG, "vf_tune_set: threads must be 512 or 1024");
    g_f32_threads.store(value);
    return VF_OK;
  }
  if (key == VF_TUNE_F32_BLOCKS_PER_SM) {
    if (value < 0 || value > 16) return fail(VF_ERR_ARG, "vf_tune_set: blocks per SM must be 0..16");
    g_f32_blocks_per_sm.store(value);
    return VF_OK;
  }
  if (key == VF_TUNE_F32_HIST_COPIES) {
    if (value != 0) return fail(VF_ERR_ARG, "vf_tune_set: the histogram layout must be 0 (joint pair tables)");
    g_f32_hist_copies.store(value);
    return VF_OK;
  }
  return fail(VF_ERR_ARG, "vf_tune_set: unknown key %d", key);
}

int vf_tune_get(int key, int* value) {
  if (!value) return fail(VF_ERR_ARG, "vf_tune_get: value is NULL");
  if (key == VF_TUNE_F32_HIST_COPIES) {
    *value = g_f32_hist_copies.load();
    return VF_OK;
  }
  if (key == VF_TUNE_F32_THREADS) {
    *value = g_f32_threads.load();
    return VF_OK;
  }
  if (key == VF_TUNE_F32_BLOCKS_PER_SM) {
    *value = g_f32_blocks_per_sm.load();
    return VF_OK;
  }
  return fail(VF_ERR_ARG, "vf_tune_get: unknown key %d", key);
}

const char* vf_last_error_string(void) { return g_err; }

int vf_preload(void) {
  // Lazily loaded kernels are loaded at their first launch; one loaded after a
  // CUDA graph exists in the process was measured to stall ~2 s on this
  // platform.  Loading them all here (a few hundred functions, once per device)
  // keeps that out of later timed or captured work.
  static std::mutex mu;
  static bool done[128] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) return fail(VF_ERR_CUDA, "vf_preload: no device");
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return VF_OK;
  cudaFuncAttributes attr;
  cudaError_t e = cudaSuccess;
  auto load = [&](const void* k) {
    if (k && e == cudaSuccess) e = cudaFuncGetAttributes(&attr, k);
  };
  for (int d = 1; d <= VF_MAX_DIM; ++d) {
    for (int integ = VF_INT_SYMGAUSS; integ <= VF_INT_SUM; ++integ) {
      load(vf::vegas_f32_kernel(d, integ, 1024));
      load(vf::vegas_f32_kernel(d, integ, 512));
      load(vf::vegas_f32_inj_kernel(d, integ, false));
    }
    for (int integ : {VF_INT_SYMGAUSS, VF_INT_PROD}) {
      load(vf::vegas_f32_tap_kernel(d, integ));
      load(vf::vegas_f32_inj_kernel(d, integ, true));
    }
  }
  for (int d = 1; d <= VF_MAX_DIM; ++d) {
    load(vf::vegas_f32_map_kernel(d, false));
    load(vf::vegas_f32_map_kernel(d, true));
  }
  for (int dmax : {4, 8, 16})
    for (int integ = VF_INT_NONE; integ <= VF_INT_SUM; ++integ) {
      load(vf::sample_kernel_f64(dmax, integ));
      load(vf::sample_kernel_f32(dmax, integ));
    }
  load((const void*)vf::vf_iteration_end_kernel);
  load((const void*)vf::vf_refine_kernel);
  load((const void*)vf::vf_consume_kernel);
  load((const void*)vf::vf_reduce_events_kernel<double>);
  load((const void*)vf::vf_reduce_events_kernel<float>);
  if (e == cudaSuccess) e = vf::preload_plus_kernels();
  if (e == cudaSuccess) e = vf::preload_batch_kernels();
  if (e == cudaSuccess) e = vf::preload_probe_kernels();
  if (e != cudaSuccess) return fail(VF_ERR_CUDA, "vf_preload: %s", cudaGetErrorString(e));
  done[dev] = true;
  return VF_OK;
}

int vf_device_info(int* sm, int* major, int* minor) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(VF_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (sm) cudaDeviceGetAttribute(sm, cudaDevAttrMultiProcessorCount, dev);
  if (major) cudaDeviceGetAttribute(major, cudaDevAttrComputeCapabilityMajor, dev);
  if (minor) cudaDeviceGetAttribute(minor, cudaDevAttrComputeCapabilityMinor, dev);
  return VF_OK;
}

int vf_sample_rows(int alg, int precision, int n_dim, int integrand, int train, int* rows) {
  if (!rows) return fail(VF_ERR_ARG, "vf_sample_rows: rows is NULL");
  if (n_dim < 1 || n_dim > VF_MAX_DIM)
    return fail(VF_ERR_UNSUPPORTED, "vf_sample_rows: n_dim=%d outside [1, %d]", n_dim, VF_MAX_DIM);
  if (precision != VF_PREC_F64 && precision != VF_PREC_F32)
    return fail(VF_ERR_ARG, "vf_sample_rows: precision=%d", precision);
  const int integ = builtin_integrand(integrand) ? integrand : VF_INT_SYMGAUSS;
  const void* k;
  int smem;
  int threads = VF_THREADS;
  const bool fast = use_vegas_f32(alg, precision, integ, false);
  if (fast) {
    threads = g_f32_threads.load();
    k = vf::vegas_f32_kernel(n_dim, integ, threads);
    smem = vf::vegas_f32_smem_bytes(n_dim, train);
  } else {
    k = sample_kernel(precision, n_dim, integ);
    const int real = precision == VF_PREC_F64 ? 8 : 4;
    smem = vf::sample_smem_bytes(real, n_dim, hist_copies_for(precision), train && alg == VF_ALG_VEGAS);
  }
  if (!k) return fail(VF_ERR_UNSUPPORTED, "vf_sample_rows: no kernel for integrand %d", integrand);
  int rc = prepare_smem(k, smem);
  if (rc) return rc;
  int per_sm = 0;
  const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem);
  if (e != cudaSuccess) return fail(VF_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
  const int sms = sm_count();
  if (sms <= 0) return fail(VF_ERR_CUDA, "no CUDA device");
  if (per_sm < 1) per_sm = 1;
  const int want = fast ? g_f32_blocks_per_sm.load() : 0;
  if (want > 0 && want < per_sm) per_sm = want;
  *rows = per_sm * sms;
  return VF_OK;
}

}  // extern "C"

namespace {

// vf_sample, with the Philox call counter optionally in device memory.
int sample_impl(int alg, int precision, const double* grid, int n_dim, long long n_events, long long ev_offset,
                double xjac, const double* xmin, const double* xdelta, double xdeltajac, const double* u_inj,
                unsigned long long seed, unsigned int call_ctr, const unsigned int* call_dev, int integrand,
                const double* params, int train, int accumulate, double* partials, int rows, int* ind_out,
                void* x_out, void* w_out, void* f_out, int* flags, void* stream) {
  if (alg != VF_ALG_VEGAS && alg != VF_ALG_PLAIN) return fail(VF_ERR_ARG, "vf_sample: alg=%d", alg);
  if (precision != VF_PREC_F64 && precision != VF_PREC_F32)
    return fail(VF_ERR_ARG, "vf_sample: precision=%d", precision);
  if (n_dim < 1 || n_dim > VF_MAX_DIM)
    return fail(VF_ERR_UNSUPPORTED, "vf_sample: n_dim=%d outside [1, %d]", n_dim, VF_MAX_DIM);
  if (n_events < 0 || ev_offset < 0) return fail(VF_ERR_ARG, "vf_sample: negative event count/offset");
  if (alg == VF_ALG_VEGAS && !grid) return fail(VF_ERR_ARG, "vf_sample: grid is NULL");
  if ((xmin == nullptr) != (xdelta == nullptr))
    return fail(VF_ERR_ARG, "vf_sample: xmin and xdelta must both be given or both NULL");
  const bool jit = integrand >= VF_INT_JIT_BASE;
  if (!builtin_integrand(integrand) && !jit) return fail(VF_ERR_ARG, "vf_sample: unknown integrand %d", integrand);
  if ((integrand == VF_INT_SYMGAUSS || integrand == VF_INT_GAUSS || integrand == VF_INT_BREIT_WIGNER) &&
      !params)
    return fail(VF_ERR_ARG, "vf_sample: integrand %d needs params", integrand);
  if (integrand != VF_INT_NONE && (!partials || rows < 1))
    return fail(VF_ERR_ARG, "vf_sample: partials/rows required when evaluating");
  if (rows < 1) rows = 1;
  const bool taps = ind_out || x_out || w_out || f_out;
  // bin indices as the only tap of an fp32 VEGAS launch with the symmetric
  // Gaussian or the product integrand: the fused sampler's parity instantiation
  const bool tap_fast = !jit && ind_out && !x_out && !w_out && !f_out && precision == VF_PREC_F32 &&
                        alg == VF_ALG_VEGAS && (integrand == VF_INT_SYMGAUSS || integrand == VF_INT_PROD);
  const bool fast = !jit && (use_vegas_f32(alg, precision, integrand, taps) || tap_fast);
  // the fp32 VEGAS map alone (no integrand, Philox uniforms): x, w, indices to HBM
  const bool map_only = !jit && precision == VF_PREC_F32 && alg == VF_ALG_VEGAS && integrand == VF_INT_NONE &&
                        !u_inj && !f_out && (x_out || w_out || ind_out);
  // fp32 VEGAS with a built-in integrand: the Philox kernel, or for injected
  // uniforms the TMA-staged kernel (VF_INJ_THREADS per block)
  const bool inj = fast && u_inj != nullptr;
  const int threads = inj ? VF_INJ_THREADS : (tap_fast ? 1024 : (fast ? g_f32_threads.load() : VF_THREADS));
  const void* k = jit        ? nullptr
                  : inj      ? vf::vegas_f32_inj_kernel(n_dim, integrand, tap_fast)
                  : tap_fast ? vf::vegas_f32_tap_kernel(n_dim, integrand)
                  : fast     ? vf::vegas_f32_kernel(n_dim, integrand, threads)
                             : sample_kernel(precision, n_dim, integrand);
  if (!k && !jit) return fail(VF_ERR_UNSUPPORTED, "vf_sample: no kernel for this configuration");

  vf::SampleArgs a;
  a.grid = grid;
  a.xmin = xmin;
  a.xdelta = xdelta;
  a.u_inj = u_inj;
  a.params = params;
  a.partials = partials;
  a.ind_out = ind_out;
  a.x_out = x_out;
  a.w_out = w_out;
  a.f_out = f_out;
  a.flags = flags;
  a.n_events = n_events;
  a.ev_offset = ev_offset;
  a.xjac = xjac;
  a.xdeltajac = xmin ? xdeltajac : 1.0;
  a.seed = seed;
  a.call_ctr = call_ctr;
  a.n_dim = n_dim;
  a.alg = alg;
  a.train = train ? 1 : 0;
  a.accumulate = accumulate ? 1 : 0;
  a.tma_swizzle = 0;
  a.rows_total = rows;
  a.call_dev = call_dev;
  fill_philox(a, seed, call_ctr);
  if (map_only) {
    const bool with_ind = ind_out != nullptr;
    const void* km = vf::vegas_f32_map_kernel(n_dim, with_ind);
    if (!km) return fail(VF_ERR_UNSUPPORTED, "vf_sample: no map kernel for n_dim=%d", n_dim);
    const int smem_m = vf::vegas_f32_map_smem_bytes(n_dim, with_ind);
    int rc = prepare_smem(km, smem_m);
    if (rc) return rc;
    const int fit = resident_blocks(km, VF_MAP_THREADS, smem_m);
    if (fit < 1) return fail(VF_ERR_CUDA, "vf_sample: occupancy query for the map kernel failed");
    // one 32-event tile per warp at least: no more blocks than the tiles need
    const long long per_block = 32LL * vf::map_ept(n_dim, with_ind) * (VF_MAP_THREADS / 32);
    const long long need = (n_events + per_block - 1) / per_block;
    long long blocks_m = fit;
    if (need < blocks_m) blocks_m = need > 0 ? need : 1;
    void* args[] = {&a};
    const cudaError_t e =
        cudaLaunchKernel(km, dim3((unsigned)blocks_m), dim3(VF_MAP_THREADS), args, smem_m, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail(VF_ERR_LAUNCH, "vf_sample launch: %s", cudaGetErrorString(e));
    return check_launch("vf_sample (map)");
  }
  if (jit) {
    if (taps && precision == VF_PREC_F32 && alg == VF_ALG_VEGAS)
      return fail(VF_ERR_UNSUPPORTED, "vf_sample: a JIT fp32 VEGAS integrand has no per-event taps");
    int fast_jit = 0;
    a.hist_copies = 0;
    const int rc = vf::jit_launch(integrand, alg, precision, n_dim, &a, rows, a.train, stream, &fast_jit,
                                  &a.hist_copies);
    (void)fast_jit;
    return rc ? rc : check_launch("vf_sample (JIT)");
  }
  int smem;
  int blocks = rows;
  if (fast) {
    a.hist_copies = 0;
    if (inj) {
      // injected uniforms: TMA tiles of VF_INJ_ROWS rows into each warp's
      // stage ring when the array allows it
      a.tma_swizzle = encode_uniform_tiles(a, u_inj, n_events, n_dim, VF_INJ_ROWS);
      smem = vf::vegas_f32_inj_smem_bytes(n_dim, a.train, a.tma_swizzle != 0);
    } else {
      smem = vf::vegas_f32_smem_bytes(n_dim, a.train);
    }
    // the grid is capped at the blocks resident at once: fewer than the
    // caller's rows when they were counted for another shape (the kernel clears
    // the rows it does not own)
    int rc = prepare_smem(k, smem);
    if (rc) return rc;
    const int fit = resident_blocks(k, threads, smem);
    if (fit < 1) return fail(VF_ERR_CUDA, "vf_sample: occupancy query for the fp32 sampler failed");
    if (fit < blocks) blocks = fit;
  } else {
    a.hist_copies = hist_copies_for(precision);
    const int real = precision == VF_PREC_F64 ? 8 : 4;
    smem = vf::sample_smem_bytes(real, n_dim, a.hist_copies, a.train && alg == VF_ALG_VEGAS);
  }
  int rc = prepare_smem(k, smem);
  if (rc) return rc;
  void* args[] = {&a};
  const cudaError_t e =
      cudaLaunchKernel(k, dim3(blocks), dim3(threads), args, smem, (cudaStream_t)stream);
  if (e != cudaSuccess) return fail(VF_ERR_LAUNCH, "vf_sample launch: %s", cudaGetErrorString(e));
  return check_launch("vf_sample");
}

}  // namespace

extern "C" {

int vf_sample(int alg, int precision, const double* grid, int n_dim, long long n_events,
              long long ev_offset, double xjac, const double* xmin, const double* xdelta,
              double xdeltajac, const double* u_inj, unsigned long long seed,
              unsigned int call_ctr, int integrand, const double* params, int train,
              int accumulate, double* partials, int rows, int* ind_out, void* x_out,
              void* w_out, void* f_out, int* flags, void* stream) {
  return sample_impl(alg, precision, grid, n_dim, n_events, ev_offset, xjac, xmin, xdelta, xdeltajac, u_inj, seed,
                     call_ctr, nullptr, integrand, params, train, accumulate, partials, rows, ind_out, x_out, w_out,
                     f_out, flags, stream);
}

int vf_reduce_events(int precision, const void* f, const void* w, const int* ind,
                     long long n_events, int n_dim, int n_out, int main_dim, int train,
                     int accumulate, double* partials, int rows, int* flags, void* stream) {
  if (!f || !w || !partials || rows < 1) return fail(VF_ERR_ARG, "vf_reduce_events: NULL buffer");
  if (n_dim < 1 || n_dim > VF_MAX_DIM) return fail(VF_ERR_UNSUPPORTED, "vf_reduce_events: n_dim=%d", n_dim);
  if (n_out < 1 || main_dim < 0 || main_dim >= n_out)
    return fail(VF_ERR_ARG, "vf_reduce_events: n_out=%d main_dim=%d", n_out, main_dim);
  if (train && !ind) return fail(VF_ERR_ARG, "vf_reduce_events: ind required when train");
  if (n_events < 0) return fail(VF_ERR_ARG, "vf_reduce_events: negative n_events");
  vf::ReduceArgs a;
  a.f = f;
  a.w = w;
  a.ind = ind;
  a.partials = partials;
  a.flags = flags;
  a.n_events = n_events;
  a.n_dim = n_dim;
  a.n_out = n_out;
  a.main_dim = main_dim;
  a.train = train ? 1 : 0;
  a.accumulate = accumulate ? 1 : 0;
  const int smem = (n_dim * VF_BINS + 16) * (int)sizeof(double);
  if (precision == VF_PREC_F64)
    vf::vf_reduce_events_kernel<double><<<rows, 256, smem, (cudaStream_t)stream>>>(a);
  else if (precision == VF_PREC_F32)
    vf::vf_reduce_events_kernel<float><<<rows, 256, smem, (cudaStream_t)stream>>>(a);
  else
    return fail(VF_ERR_ARG, "vf_reduce_events: precision=%d", precision);
  return check_launch("vf_reduce_events");
}

}  // extern "C"

namespace {

// vf_iteration_end, with the iteration index (and the call counter it advances)
// optionally in device memory.
int iteration_end_impl(const double* partials, int rows, int n_dim, int n_out, int train, double n_events,
                       double alpha, double* grid, double* hist_out, double* sums_out, double* history, double* avg,
                       int iter, int* iter_dev, unsigned int* call_dev, int hist_cap, int* flags, void* stream) {
  if (!partials || rows < 1 || !history || !avg || iter < 0)
    return fail(VF_ERR_ARG, "vf_iteration_end: NULL buffer or bad rows/iter");
  if (n_dim < 1 || n_dim > VF_MAX_DIM) return fail(VF_ERR_UNSUPPORTED, "vf_iteration_end: n_dim=%d", n_dim);
  if (n_out < 1) return fail(VF_ERR_ARG, "vf_iteration_end: n_out=%d", n_out);
  if (train < 0 || train > 2) return fail(VF_ERR_ARG, "vf_iteration_end: train=%d (0, 1 or 2)", train);
  if (train && !grid) return fail(VF_ERR_ARG, "vf_iteration_end: grid required when train");
  vf::IterEndArgs a;
  a.partials = partials;
  a.grid = grid;
  a.hist_out = hist_out;
  a.sums_out = sums_out;
  a.history = history;
  a.avg = avg;
  a.flags = flags;
  a.n_events = n_events;
  a.alpha = alpha;
  a.rows = rows;
  a.n_dim = n_dim;
  a.n_out = n_out;
  a.train = train == 2 ? 2 : (train ? 1 : 0);
  a.iter = iter;
  a.iter_dev = iter_dev;
  a.call_dev = call_dev;
  a.hist_cap = hist_cap;
  const int clusters = (a.train || hist_out) ? n_dim + 1 : 1;
  {
    // the samplers run with the largest shared-memory carveout; the same
    // preference here spares an L1/shared reconfiguration between the launches
    static std::once_flag once;
    std::call_once(once, [] {
      cudaFuncSetAttribute(vf::vf_iteration_end_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                           cudaSharedmemCarveoutMaxShared);
    });
  }
  vf::vf_iteration_end_kernel<<<clusters * VF_END_CLUSTER, VF_END_THREADS, 0, (cudaStream_t)stream>>>(a);
  return check_launch("vf_iteration_end");
}

}  // namespace

extern "C" {

int vf_iteration_end(const double* partials, int rows, int n_dim, int n_out, int train,
                     double n_events, double alpha, double* grid, double* hist_out,
                     double* sums_out, double* history, double* avg, int iter, int* flags,
                     void* stream) {
  return iteration_end_impl(partials, rows, n_dim, n_out, train, n_events, alpha, grid, hist_out, sums_out, history,
                            avg, iter, nullptr, nullptr, 0, flags, stream);
}

int vf_iteration_dev(int alg, int precision, double* grid, int n_dim, long long n_events, double xjac,
                     const double* xmin, const double* xdelta, double xdeltajac, unsigned long long seed,
                     unsigned int* call_dev, int* iter_dev, int integrand, const double* params, int train,
                     double alpha, double* partials, int rows, double* history, int hist_cap, double* avg,
                     int* flags, void* stream) {
  if (!call_dev || !iter_dev) return fail(VF_ERR_ARG, "vf_iteration_dev: call_dev and iter_dev are required");
  if (hist_cap < 1) return fail(VF_ERR_ARG, "vf_iteration_dev: hist_cap=%d", hist_cap);
  if (integrand == VF_INT_NONE) return fail(VF_ERR_ARG, "vf_iteration_dev: needs an integrand");
  const int tr = alg == VF_ALG_VEGAS && train ? (precision == VF_PREC_F32 ? 2 : 1) : 0;
  int rc = sample_impl(alg, precision, grid, n_dim, n_events, 0, xjac, xmin, xdelta, xdeltajac, nullptr, seed, 0,
                       call_dev, integrand, params, tr != 0, 0, partials, rows, nullptr, nullptr, nullptr, nullptr, flags,
                       stream);
  if (rc) return rc;
  return iteration_end_impl(partials, rows, n_dim, 1, tr, (double)n_events, alpha, grid, nullptr, nullptr, history,
                            avg, 0, iter_dev, call_dev, hist_cap, flags, stream);
}

int vf_refine_grid(double* grid, const double* hist, int n_dim, double alpha, int* flags,
                   void* stream) {
  if (!grid || !hist) return fail(VF_ERR_ARG, "vf_refine_grid: NULL buffer");
  if (n_dim < 1 || n_dim > 4096) return fail(VF_ERR_ARG, "vf_refine_grid: n_dim=%d", n_dim);
  vf::vf_refine_kernel<<<n_dim, 64, 0, (cudaStream_t)stream>>>(grid, hist, alpha, flags);
  return check_launch("vf_refine_grid");
}

int vf_philox_uniforms(unsigned long long seed, unsigned int call_ctr, unsigned int word3, long long ev_offset,
                       long long n, int n_dim, double* u_out, void* stream) {
  if (!u_out && n > 0) return fail(VF_ERR_ARG, "vf_philox_uniforms: u_out is NULL");
  if (n_dim < 1 || n_dim > VF_MAX_DIM) return fail(VF_ERR_UNSUPPORTED, "vf_philox_uniforms: n_dim=%d", n_dim);
  if (n < 0 || ev_offset < 0) return fail(VF_ERR_ARG, "vf_philox_uniforms: negative count/offset");
  if (n == 0) return VF_OK;
  vf::SampleArgs a;
  fill_philox(a, seed, call_ctr);
  long long blocks = (n + 255) / 256;
  const int cap = 8 * (sm_count() > 0 ? sm_count() : 1);
  if (blocks > cap) blocks = cap;
  vf::vf_philox_uniforms_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(a.rk, call_ctr << 4, word3, ev_offset,
                                                                               n, n_dim, u_out);
  return check_launch("vf_philox_uniforms");
}

int vf_consume_array_into_indices(const double* input, const int* indices, long long n,
                                  int result_size, double* out, int* flags, void* stream) {
  if (!out || result_size < 1) return fail(VF_ERR_ARG, "vf_consume_array_into_indices: bad output");
  if (n > 0 && (!input || !indices)) return fail(VF_ERR_ARG, "vf_consume_array_into_indices: NULL input");
  if (result_size > 12288) return fail(VF_ERR_UNSUPPORTED, "result_size %d > 12288", result_size);
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * result_size, (cudaStream_t)stream);
  if (e != cudaSuccess) return fail(VF_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
  if (n == 0) return VF_OK;
  const int smem = result_size * (int)sizeof(double);
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(vf::vf_consume_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return fail(VF_ERR_CUDA, "smem attribute: %s", cudaGetErrorString(e));
  }
  long long blocks = (n + 255) / 256;
  const int cap = 4 * (sm_count() > 0 ? sm_count() : 1);
  if (blocks > cap) blocks = cap;
  vf::vf_consume_kernel<<<(int)blocks, 256, smem, (cudaStream_t)stream>>>(input, indices, n, result_size,
                                                                           out, flags);
  return check_launch("vf_consume_array_into_indices");
}

}  // extern "C"
