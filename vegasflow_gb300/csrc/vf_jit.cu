// NVRTC-compiled user integrands.
//
// A user integrand is CUDA source defining a device function
//     vf_real f(const vf_real* x, int n_dim, vf_real weight, const double* params)
// (vf_real = the sampler's precision, typedef'd before the source).  It is
// compiled together with the sampler headers (embedded in the library) into a
// sampler kernel specialised for the integrand: the fp32 VEGAS kernel on the
// exact dimension count, the generic sampler for float64 and plain MC, the
// VEGAS+ samplers, or the batched sampler of a dimension class.
// The CUBIN is built for sm_103a and loaded with the driver API; launches go
// through vf_sample with the returned integrand id.
#include <cuda.h>
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <mutex>
#include <string>
#include <vector>

#include "vegasflow_gb300.h"
#include "vf_internal.h"
#include "vf_batch_sampler.cuh"
#include "vf_jit_sources.h"
#include "vf_plus_f32.cuh"
#include "vf_plus_sampler.cuh"
#include "vf_vegas_f32.cuh"

namespace {

// Driver entry points, resolved through the runtime (no link-time dependency on
// the driver library, so the library loads on machines without a GPU driver).
typedef CUresult (*PfnModuleLoadData)(CUmodule*, const void*);
typedef CUresult (*PfnModuleGetFunction)(CUfunction*, CUmodule, const char*);
typedef CUresult (*PfnLaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                                    unsigned, CUstream, void**, void**);
typedef CUresult (*PfnFuncSetAttribute)(CUfunction, CUfunction_attribute, int);

struct Driver {
  PfnModuleLoadData module_load_data = nullptr;
  PfnModuleGetFunction module_get_function = nullptr;
  PfnLaunchKernel launch_kernel = nullptr;
  PfnFuncSetAttribute func_set_attribute = nullptr;
  bool ok = false;
};

const Driver& driver() {
  static Driver d;
  static std::once_flag once;
  std::call_once(once, [] {
    auto get = [](const char* name, void** fn) {
      cudaDriverEntryPointQueryResult q;
      return cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
             q == cudaDriverEntryPointSuccess && *fn != nullptr;
    };
    d.ok = get("cuModuleLoadData", reinterpret_cast<void**>(&d.module_load_data)) &&
           get("cuModuleGetFunction", reinterpret_cast<void**>(&d.module_get_function)) &&
           get("cuLaunchKernel", reinterpret_cast<void**>(&d.launch_kernel)) &&
           get("cuFuncSetAttribute", reinterpret_cast<void**>(&d.func_set_attribute));
  });
  return d;
}

struct JitKernel {
  CUmodule module = nullptr;
  CUfunction fn = nullptr;       // the sampler (VEGAS+: the float64 / tap-writing one; fp32 VEGAS: the
                                 // Philox kernel, 1024 threads per block)
  CUfunction fn_fast = nullptr;  // VEGAS+ in fp32: the float32 sampler for Philox uniforms; fp32 VEGAS:
                                 // the kernel for injected uniforms (1024 threads per block)
  int alg = 0, precision = 0, n_dim = 0, fast = 0, smem_set = 0, smem_set_fast = 0;
};

std::mutex g_mu;
std::vector<JitKernel> g_kernels;

// The program around a user integrand and the kernels to take from it: for
// VEGAS and plain MC one sampler; for VEGAS+ the generic sampler and, in fp32,
// also the float32 one.
std::string program_text(const char* source, const char* func_name, int alg, int precision, int n_dim,
                         std::vector<std::string>* exprs) {
  const bool fast = precision == VF_PREC_F32 && alg == VF_ALG_VEGAS;
  const char* real = precision == VF_PREC_F64 ? "double" : "float";
  std::string src = "#define VF_JIT_USER 1\n";
  src += std::string("typedef ") + real + " vf_real;\n";
  src += source;
  // the samplers call the user function through a global-scope wrapper with an
  // unusual name: a kernel local (f, x, w, ...) cannot shadow it there
  src += "\n__device__ __forceinline__ vf_real vf_user_integrand_call_(const vf_real* vf_x_, int vf_n_, "
         "vf_real vf_w_, const double* vf_p_) { return " +
         std::string(func_name) + "(vf_x_, vf_n_, vf_w_, vf_p_); }\n";
  src += "#define VF_USER_FN vf_user_integrand_call_\n";
  exprs->clear();
  if (alg == VF_ALG_BATCH) {
    src += "#include \"vf_batch_sampler.cuh\"\n";
    exprs->push_back("vf::vf_batch_sample_kernel<" + std::to_string(n_dim <= 8 ? 8 : 16) + ", true>");
  } else if (alg == VF_ALG_PLUS) {
    src += "#include \"vf_plus_sampler.cuh\"\n";
    exprs->push_back(std::string("vf::vf_plus_kernel<") + real + ", " + std::to_string(vf::dim_bucket(n_dim)) +
                     ", 99>");
    if (precision == VF_PREC_F32) {
      src += "#include \"vf_plus_f32.cuh\"\n";
      exprs->push_back("vf::vf_plus_f32_kernel<" + std::to_string(n_dim) + ", 99>");
    }
  } else if (fast) {
    src += "#include \"vf_vegas_f32.cuh\"\n";
    exprs->push_back("vf::vf_vegas_f32_kernel<" + std::to_string(n_dim) + ", 99, 1024>");
    exprs->push_back("vf::vf_vegas_f32_inj_kernel<" + std::to_string(n_dim) + ", 99>");
  } else {
    src += "#include \"vf_sample.cuh\"\n";
    exprs->push_back(std::string("vf::vf_sample_kernel<") + real + ", " + std::to_string(vf::dim_bucket(n_dim)) +
                     ", 99>");
  }
  return src;
}

// Compile; on success returns the CUBIN and the lowered kernel names.
int compile(const char* source, const char* func_name, int alg, int precision, int n_dim, std::vector<char>* cubin,
            std::vector<std::string>* lowered, std::string* log) {
  if (!source || !func_name || !*func_name) return VF_ERR_ARG;
  if (n_dim < 1 || n_dim > VF_MAX_DIM) return VF_ERR_UNSUPPORTED;
  if ((alg != VF_ALG_VEGAS && alg != VF_ALG_PLAIN && alg != VF_ALG_PLUS && alg != VF_ALG_BATCH) ||
      (precision != VF_PREC_F64 && precision != VF_PREC_F32) || (alg == VF_ALG_BATCH && precision != VF_PREC_F32))
    return VF_ERR_ARG;
  std::vector<std::string> exprs;
  const std::string src = program_text(source, func_name, alg, precision, n_dim, &exprs);
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, src.c_str(), "vf_user_integrand.cu", kJitHeaderCount, kJitHeaderSources,
                         kJitHeaderNames) != NVRTC_SUCCESS)
    return VF_ERR_JIT;
  for (const std::string& e : exprs) nvrtcAddNameExpression(prog, e.c_str());
  const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo"};
  const nvrtcResult rc = nvrtcCompileProgram(prog, 3, opts);
  size_t log_size = 0;
  nvrtcGetProgramLogSize(prog, &log_size);
  if (log && log_size > 1) {
    log->resize(log_size);
    nvrtcGetProgramLog(prog, &(*log)[0]);
  }
  if (rc != NVRTC_SUCCESS) {
    nvrtcDestroyProgram(&prog);
    return VF_ERR_JIT;
  }
  if (lowered) {
    lowered->clear();
    for (const std::string& e : exprs) {
      const char* name = nullptr;
      nvrtcGetLoweredName(prog, e.c_str(), &name);
      lowered->push_back(name ? name : "");
    }
  }
  if (cubin) {
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    cubin->resize(n);
    nvrtcGetCUBIN(prog, cubin->data());
  }
  nvrtcDestroyProgram(&prog);
  return VF_OK;
}

}  // namespace

namespace vf {

// Launch a VEGAS+ JIT kernel for vf_plus_sample (declared in vf_internal.h):
// the float32 one when `use_fast` (fp32, Philox uniforms, no taps), else the
// generic one.
int jit_launch_plus(int integrand_id, int precision, int n_dim, void* args, int rows, int train, bool use_fast,
                    void* stream) {
  JitKernel k;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    const int idx = integrand_id - VF_INT_JIT_BASE;
    if (idx < 0 || idx >= (int)g_kernels.size()) return set_error(VF_ERR_ARG, "unknown JIT integrand id");
    k = g_kernels[idx];
  }
  if (k.alg != VF_ALG_PLUS || k.precision != precision || k.n_dim != n_dim)
    return set_error(VF_ERR_ARG, "JIT integrand was compiled for another algorithm, precision or n_dim");
  const bool fast = use_fast && k.fn_fast != nullptr;
  const CUfunction fn = fast ? k.fn_fast : k.fn;
  const int smem = fast ? plus_f32_smem_bytes(n_dim, train)
                        : plus_smem_bytes(precision == VF_PREC_F64 ? 8 : 4, n_dim, train);
  const Driver& drv = driver();
  if (!drv.ok) return set_error(VF_ERR_CUDA, "CUDA driver entry points unavailable");
  if (smem > 48 * 1024 && (fast ? k.smem_set_fast : k.smem_set) < smem) {
    if (drv.func_set_attribute(fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, smem) != CUDA_SUCCESS)
      return set_error(VF_ERR_CUDA, "cuFuncSetAttribute for a JIT kernel failed");
    std::lock_guard<std::mutex> lock(g_mu);
    JitKernel& kk = g_kernels[integrand_id - VF_INT_JIT_BASE];
    (fast ? kk.smem_set_fast : kk.smem_set) = smem;
  }
  void* params[] = {args};
  const CUresult r = drv.launch_kernel(fn, rows, 1, 1, VF_THREADS, 1, 1, smem, (CUstream)stream, params, nullptr);
  if (r != CUDA_SUCCESS) return set_error(VF_ERR_LAUNCH, "cuLaunchKernel failed for a JIT kernel");
  return VF_OK;
}

// Launch a batched JIT sampler for vf_batch_sample_jit (declared in vf_internal.h).
int jit_launch_batch(int integrand_id, int max_dim, void* args, int blocks, int smem, void* stream) {
  JitKernel k;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    const int idx = integrand_id - VF_INT_JIT_BASE;
    if (idx < 0 || idx >= (int)g_kernels.size()) return set_error(VF_ERR_ARG, "unknown JIT integrand id");
    k = g_kernels[idx];
  }
  if (k.alg != VF_ALG_BATCH) return set_error(VF_ERR_ARG, "JIT integrand was not compiled for VF_ALG_BATCH");
  if (max_dim > (k.n_dim <= 8 ? 8 : 16))
    return set_error(VF_ERR_ARG, "JIT integrand was compiled for integrals of fewer dimensions");
  const Driver& drv = driver();
  if (!drv.ok) return set_error(VF_ERR_CUDA, "CUDA driver entry points unavailable");
  if (smem > 48 * 1024 && k.smem_set < smem) {
    if (drv.func_set_attribute(k.fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, smem) != CUDA_SUCCESS)
      return set_error(VF_ERR_CUDA, "cuFuncSetAttribute for a JIT kernel failed");
    std::lock_guard<std::mutex> lock(g_mu);
    JitKernel& kk = g_kernels[integrand_id - VF_INT_JIT_BASE];
    if (kk.smem_set < smem) kk.smem_set = smem;
  }
  void* params[] = {args};
  const CUresult r = drv.launch_kernel(k.fn, blocks, 1, 1, VF_THREADS, 1, 1, smem, (CUstream)stream, params, nullptr);
  if (r != CUDA_SUCCESS) return set_error(VF_ERR_LAUNCH, "cuLaunchKernel failed for a JIT kernel");
  return VF_OK;
}

// Launch a JIT kernel for vf_sample (declared in vf_internal.h).
int jit_launch(int integrand_id, int alg, int precision, int n_dim, void* args, int rows, int train, void* stream,
               int* fast_out, int* hist_copies_inout) {
  JitKernel k;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    const int idx = integrand_id - VF_INT_JIT_BASE;
    if (idx < 0 || idx >= (int)g_kernels.size()) return set_error(VF_ERR_ARG, "unknown JIT integrand id");
    k = g_kernels[idx];
  }
  if (k.alg != alg || k.precision != precision || k.n_dim != n_dim)
    return set_error(VF_ERR_ARG, "JIT integrand was compiled for another algorithm, precision or n_dim");
  *fast_out = k.fast;
  int smem;
  unsigned threads = VF_THREADS;
  int blocks = rows;
  // fp32 VEGAS: the injected-uniform kernel when uniforms are injected
  const bool inj = k.fast && static_cast<const SampleArgs*>(args)->u_inj != nullptr;
  const CUfunction fn = inj ? k.fn_fast : k.fn;
  if (k.fast) {
    // both fp32 VEGAS kernels run 1024-thread blocks, one per SM (64 registers
    // per thread); the kernel clears the caller's rows beyond its grid
    *hist_copies_inout = 0;
    smem = inj ? vegas_f32_inj_smem_bytes(n_dim, train) : vegas_f32_smem_bytes(n_dim, train);
    threads = 1024;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0 && sms < blocks)
      blocks = sms;
  } else {
    *hist_copies_inout = precision == VF_PREC_F32 ? 8 : 1;
    smem = sample_smem_bytes(precision == VF_PREC_F64 ? 8 : 4, n_dim, *hist_copies_inout,
                             train && alg == VF_ALG_VEGAS);
  }
  const Driver& drv = driver();
  if (!drv.ok) return set_error(VF_ERR_CUDA, "CUDA driver entry points unavailable");
  const int have = inj ? k.smem_set_fast : k.smem_set;
  if (smem > 48 * 1024 && have < smem) {  // once per size: no attribute call in later (captured) launches
    if (drv.func_set_attribute(fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, smem) != CUDA_SUCCESS)
      return set_error(VF_ERR_CUDA, "cuFuncSetAttribute for a JIT kernel failed");
    std::lock_guard<std::mutex> lock(g_mu);
    JitKernel& kk = g_kernels[integrand_id - VF_INT_JIT_BASE];
    int& set = inj ? kk.smem_set_fast : kk.smem_set;
    if (set < smem) set = smem;
  }
  void* params[] = {args};
  const CUresult r =
      drv.launch_kernel(fn, blocks, 1, 1, threads, 1, 1, smem, (CUstream)stream, params, nullptr);
  if (r != CUDA_SUCCESS) return set_error(VF_ERR_LAUNCH, "cuLaunchKernel failed for a JIT kernel");
  return VF_OK;
}

}  // namespace vf

extern "C" {

int vf_jit_check(const char* source, const char* func_name, int alg, int precision, int n_dim, char* log,
                 int log_size) {
  std::string lg;
  const int rc = compile(source, func_name, alg, precision, n_dim, nullptr, nullptr, &lg);
  if (log && log_size > 0) {
    const size_t n = lg.size() < (size_t)log_size - 1 ? lg.size() : (size_t)log_size - 1;
    lg.copy(log, n);
    log[n] = 0;
  }
  if (rc == VF_ERR_JIT) return vf::set_error(rc, ("NVRTC: " + lg).c_str());
  if (rc) return vf::set_error(rc, "vf_jit_check: bad arguments");
  return VF_OK;
}

int vf_jit_integrand(const char* source, const char* func_name, int alg, int precision, int n_dim,
                     int* integrand_id) {
  if (!integrand_id) return vf::set_error(VF_ERR_ARG, "vf_jit_integrand: integrand_id is NULL");
  std::vector<char> cubin;
  std::vector<std::string> lowered;
  std::string lg;
  int rc = compile(source, func_name, alg, precision, n_dim, &cubin, &lowered, &lg);
  if (rc == VF_ERR_JIT) return vf::set_error(rc, ("NVRTC: " + lg).c_str());
  if (rc) return vf::set_error(rc, "vf_jit_integrand: bad arguments");
  if (cudaFree(nullptr) != cudaSuccess)  // make the device's primary context current
    return vf::set_error(VF_ERR_CUDA, "vf_jit_integrand: no CUDA context");
  const Driver& drv = driver();
  if (!drv.ok) return vf::set_error(VF_ERR_CUDA, "vf_jit_integrand: CUDA driver entry points unavailable");
  JitKernel k;
  if (drv.module_load_data(&k.module, cubin.data()) != CUDA_SUCCESS)
    return vf::set_error(VF_ERR_JIT, "vf_jit_integrand: cuModuleLoadData failed");
  if (lowered.empty() || drv.module_get_function(&k.fn, k.module, lowered[0].c_str()) != CUDA_SUCCESS)
    return vf::set_error(VF_ERR_JIT, "vf_jit_integrand: kernel not found in the module");
  if (lowered.size() > 1 && drv.module_get_function(&k.fn_fast, k.module, lowered[1].c_str()) != CUDA_SUCCESS)
    return vf::set_error(VF_ERR_JIT, "vf_jit_integrand: kernel not found in the module");
  k.alg = alg;
  k.precision = precision;
  k.n_dim = n_dim;
  k.fast = precision == VF_PREC_F32 && alg == VF_ALG_VEGAS;
  std::lock_guard<std::mutex> lock(g_mu);
  g_kernels.push_back(k);
  *integrand_id = VF_INT_JIT_BASE + (int)g_kernels.size() - 1;
  return VF_OK;
}

}  // extern "C"
