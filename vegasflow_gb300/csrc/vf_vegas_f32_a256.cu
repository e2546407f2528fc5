// Ahead-of-time instantiations of the fp32 VEGAS sampler: dimensions 1-8, 256 threads per block.
#include "vf_internal.h"
#include "vf_vegas_f32.cuh"

namespace vf {

template <int D>
static const void* pick(int integrand) {
  switch (integrand) {
    case VF_INT_SYMGAUSS: return (const void*)vf_vegas_f32_kernel<D, VF_INT_SYMGAUSS, 256>;
    case VF_INT_GAUSS: return (const void*)vf_vegas_f32_kernel<D, VF_INT_GAUSS, 256>;
    case VF_INT_BREIT_WIGNER: return (const void*)vf_vegas_f32_kernel<D, VF_INT_BREIT_WIGNER, 256>;
    case VF_INT_PROD: return (const void*)vf_vegas_f32_kernel<D, VF_INT_PROD, 256>;
    case VF_INT_SUM: return (const void*)vf_vegas_f32_kernel<D, VF_INT_SUM, 256>;
    default: return nullptr;
  }
}

const void* vegas_f32_kernel_a256(int n_dim, int integrand) {
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
