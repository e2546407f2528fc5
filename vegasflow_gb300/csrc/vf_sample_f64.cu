// Ahead-of-time instantiations of the double sampler for the built-in integrands.
#include "vf_sample.cuh"
#include "vf_internal.h"

namespace vf {

template <int DMAX>
static const void* pick(int integrand) {
  switch (integrand) {
    case VF_INT_NONE: return (const void*)vf_sample_kernel<double, DMAX, VF_INT_NONE>;
    case VF_INT_SYMGAUSS: return (const void*)vf_sample_kernel<double, DMAX, VF_INT_SYMGAUSS>;
    case VF_INT_GAUSS: return (const void*)vf_sample_kernel<double, DMAX, VF_INT_GAUSS>;
    case VF_INT_BREIT_WIGNER: return (const void*)vf_sample_kernel<double, DMAX, VF_INT_BREIT_WIGNER>;
    case VF_INT_PROD: return (const void*)vf_sample_kernel<double, DMAX, VF_INT_PROD>;
    case VF_INT_SUM: return (const void*)vf_sample_kernel<double, DMAX, VF_INT_SUM>;
    default: return nullptr;
  }
}

const void* sample_kernel_f64(int dmax, int integrand) {
  switch (dmax) {
    case 4: return pick<4>(integrand);
    case 8: return pick<8>(integrand);
    case 16: return pick<16>(integrand);
    default: return nullptr;
  }
}

}  // namespace vf
