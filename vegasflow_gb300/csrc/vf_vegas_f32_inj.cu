// Ahead-of-time instantiations of the fp32 VEGAS sampler for injected float64
// uniforms (every built-in integrand; the parity instantiation writing bin
// indices for the symmetric Gaussian and the product integrand), for one range
// of dimension counts: build.py compiles this file once per (VF_INST_DLO,
// VF_INST_DHI) variant.
#include "vf_internal.h"
#include "vf_vegas_f32.cuh"

#if !defined(VF_INST_DLO) || !defined(VF_INST_DHI)
#error "compile with -DVF_INST_DLO=... -DVF_INST_DHI=..."
#endif

#define VF_CAT3_(a, b, c) a##b##_##c
#define VF_CAT3(a, b, c) VF_CAT3_(a, b, c)

namespace vf {

namespace {

template <int D>
const void* pick(int integrand, bool tap) {
  if (tap) {
    switch (integrand) {
      case VF_INT_SYMGAUSS: return (const void*)vf_vegas_f32_inj_kernel<D, VF_INT_SYMGAUSS, true>;
      case VF_INT_PROD: return (const void*)vf_vegas_f32_inj_kernel<D, VF_INT_PROD, true>;
      default: return nullptr;
    }
  }
  switch (integrand) {
    case VF_INT_SYMGAUSS: return (const void*)vf_vegas_f32_inj_kernel<D, VF_INT_SYMGAUSS>;
    case VF_INT_GAUSS: return (const void*)vf_vegas_f32_inj_kernel<D, VF_INT_GAUSS>;
    case VF_INT_BREIT_WIGNER: return (const void*)vf_vegas_f32_inj_kernel<D, VF_INT_BREIT_WIGNER>;
    case VF_INT_PROD: return (const void*)vf_vegas_f32_inj_kernel<D, VF_INT_PROD>;
    case VF_INT_SUM: return (const void*)vf_vegas_f32_inj_kernel<D, VF_INT_SUM>;
    default: return nullptr;
  }
}

template <int D>
const void* pick_range(int n_dim, int integrand, bool tap) {
  if constexpr (D > VF_INST_DHI)
    return nullptr;
  else
    return n_dim == D ? pick<D>(integrand, tap) : pick_range<D + 1>(n_dim, integrand, tap);
}

}  // namespace

const void* VF_CAT3(vegas_f32_inj_kernel_d, VF_INST_DLO, VF_INST_DHI)(int n_dim, int integrand, bool tap) {
  return pick_range<VF_INST_DLO>(n_dim, integrand, tap);
}

}  // namespace vf
