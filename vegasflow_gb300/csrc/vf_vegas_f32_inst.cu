// Ahead-of-time instantiations of the fp32 VEGAS Philox sampler for one block
// size and one range of dimension counts, every built-in integrand.  build.py
// compiles this file once per (VF_INST_THREADS, VF_INST_DLO, VF_INST_DHI)
// variant, so the instantiations build in parallel.
#include "vf_internal.h"
#include "vf_vegas_f32.cuh"

#if !defined(VF_INST_THREADS) || !defined(VF_INST_DLO) || !defined(VF_INST_DHI)
#error "compile with -DVF_INST_THREADS=... -DVF_INST_DLO=... -DVF_INST_DHI=..."
#endif

#define VF_CAT4_(a, b, c, d) a##b##_##c##_##d
#define VF_CAT4(a, b, c, d) VF_CAT4_(a, b, c, d)

namespace vf {

namespace {

template <int D>
const void* pick(int integrand) {
  switch (integrand) {
    case VF_INT_SYMGAUSS: return (const void*)vf_vegas_f32_kernel<D, VF_INT_SYMGAUSS, VF_INST_THREADS>;
    case VF_INT_GAUSS: return (const void*)vf_vegas_f32_kernel<D, VF_INT_GAUSS, VF_INST_THREADS>;
    case VF_INT_BREIT_WIGNER: return (const void*)vf_vegas_f32_kernel<D, VF_INT_BREIT_WIGNER, VF_INST_THREADS>;
    case VF_INT_PROD: return (const void*)vf_vegas_f32_kernel<D, VF_INT_PROD, VF_INST_THREADS>;
    case VF_INT_SUM: return (const void*)vf_vegas_f32_kernel<D, VF_INT_SUM, VF_INST_THREADS>;
    default: return nullptr;
  }
}

template <int D>
const void* pick_range(int n_dim, int integrand) {
  if constexpr (D > VF_INST_DHI)
    return nullptr;
  else
    return n_dim == D ? pick<D>(integrand) : pick_range<D + 1>(n_dim, integrand);
}

}  // namespace

const void* VF_CAT4(vegas_f32_kernel_t, VF_INST_THREADS, VF_INST_DLO, VF_INST_DHI)(int n_dim, int integrand) {
  return pick_range<VF_INST_DLO>(n_dim, integrand);
}

}  // namespace vf
