// Ahead-of-time instantiations of the fp32 VEGAS sampler, dimensions 1-8.
#include "vf_internal.h"
#include "vf_vegas_f32.cuh"

namespace vf {

template <int D>
static const void* pick(int integrand) {
  switch (integrand) {
    case VF_INT_SYMGAUSS: return (const void*)vf_vegas_f32_kernel<D, VF_INT_SYMGAUSS>;
    case VF_INT_GAUSS: return (const void*)vf_vegas_f32_kernel<D, VF_INT_GAUSS>;
    case VF_INT_BREIT_WIGNER: return (const void*)vf_vegas_f32_kernel<D, VF_INT_BREIT_WIGNER>;
    case VF_INT_PROD: return (const void*)vf_vegas_f32_kernel<D, VF_INT_PROD>;
    case VF_INT_SUM: return (const void*)vf_vegas_f32_kernel<D, VF_INT_SUM>;
    default: return nullptr;
  }
}

const void* vegas_f32_kernel_a(int n_dim, int integrand) {
  switch (n_dim) {
    case 1: return pick<1>(integrand);
    case 2: return pick<2>(integrand);
    case 3: return pick<3>(integrand);
    case 4: return pick<4>(integrand);
    case 5: return pick<5>(integrand);
    case 6: return pick<6>(integrand);
    case 7: return pick<7>(integrand);
    case 8: return pick<8>(integrand);
    default: return nullptr;
  }
}

}  // namespace vf
