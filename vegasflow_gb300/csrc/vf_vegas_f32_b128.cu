// Ahead-of-time instantiations of the fp32 VEGAS sampler: dimensions 9-16, 128 threads per block.
#include "vf_internal.h"
#include "vf_vegas_f32.cuh"

namespace vf {

template <int D>
static const void* pick(int integrand) {
  switch (integrand) {
    case VF_INT_SYMGAUSS: return (const void*)vf_vegas_f32_kernel<D, VF_INT_SYMGAUSS, 128>;
    case VF_INT_GAUSS: return (const void*)vf_vegas_f32_kernel<D, VF_INT_GAUSS, 128>;
    case VF_INT_BREIT_WIGNER: return (const void*)vf_vegas_f32_kernel<D, VF_INT_BREIT_WIGNER, 128>;
    case VF_INT_PROD: return (const void*)vf_vegas_f32_kernel<D, VF_INT_PROD, 128>;
    case VF_INT_SUM: return (const void*)vf_vegas_f32_kernel<D, VF_INT_SUM, 128>;
    default: return nullptr;
  }
}

const void* vegas_f32_kernel_b128(int n_dim, int integrand) {
  switch (n_dim) {
    case 9: return pick<9>(integrand);
    case 10: return pick<10>(integrand);
    case 11: return pick<11>(integrand);
    case 12: return pick<12>(integrand);
    case 13: return pick<13>(integrand);
    case 14: return pick<14>(integrand);
    case 15: return pick<15>(integrand);
    case 16: return pick<16>(integrand);
    default: return nullptr;
  }
}

}  // namespace vf
