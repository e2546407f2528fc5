// Ahead-of-time instantiations of the fp32 VEGAS+ sampler (dimensions 1-16,
// the built-in integrands).
#include "vf_internal.h"
#include "vf_plus_f32.cuh"

namespace vf {

template <int D>
static const void* pick_plus_f32(int integrand) {
  switch (integrand) {
    case VF_INT_SYMGAUSS: return (const void*)vf_plus_f32_kernel<D, VF_INT_SYMGAUSS>;
    case VF_INT_GAUSS: return (const void*)vf_plus_f32_kernel<D, VF_INT_GAUSS>;
    case VF_INT_BREIT_WIGNER: return (const void*)vf_plus_f32_kernel<D, VF_INT_BREIT_WIGNER>;
    case VF_INT_PROD: return (const void*)vf_plus_f32_kernel<D, VF_INT_PROD>;
    case VF_INT_SUM: return (const void*)vf_plus_f32_kernel<D, VF_INT_SUM>;
    default: return nullptr;
  }
}

// the parity instantiations (bin-index and point taps), two integrands
template <int D>
static const void* pick_plus_f32_tap(int integrand) {
  switch (integrand) {
    case VF_INT_SYMGAUSS: return (const void*)vf_plus_f32_kernel<D, VF_INT_SYMGAUSS, true>;
    case VF_INT_BREIT_WIGNER: return (const void*)vf_plus_f32_kernel<D, VF_INT_BREIT_WIGNER, true>;
    default: return nullptr;
  }
}

const void* plus_f32_tap_kernel(int n_dim, int integrand) {
  switch (n_dim) {
    case 1: return pick_plus_f32_tap<1>(integrand);
    case 2: return pick_plus_f32_tap<2>(integrand);
    case 3: return pick_plus_f32_tap<3>(integrand);
    case 4: return pick_plus_f32_tap<4>(integrand);
    case 5: return pick_plus_f32_tap<5>(integrand);
    case 6: return pick_plus_f32_tap<6>(integrand);
    case 7: return pick_plus_f32_tap<7>(integrand);
    case 8: return pick_plus_f32_tap<8>(integrand);
    case 9: return pick_plus_f32_tap<9>(integrand);
    case 10: return pick_plus_f32_tap<10>(integrand);
    case 11: return pick_plus_f32_tap<11>(integrand);
    case 12: return pick_plus_f32_tap<12>(integrand);
    case 13: return pick_plus_f32_tap<13>(integrand);
    case 14: return pick_plus_f32_tap<14>(integrand);
    case 15: return pick_plus_f32_tap<15>(integrand);
    case 16: return pick_plus_f32_tap<16>(integrand);
    default: return nullptr;
  }
}

const void* plus_f32_kernel(int n_dim, int integrand) {
  switch (n_dim) {
    case 1: return pick_plus_f32<1>(integrand);
    case 2: return pick_plus_f32<2>(integrand);
    case 3: return pick_plus_f32<3>(integrand);
    case 4: return pick_plus_f32<4>(integrand);
    case 5: return pick_plus_f32<5>(integrand);
    case 6: return pick_plus_f32<6>(integrand);
    case 7: return pick_plus_f32<7>(integrand);
    case 8: return pick_plus_f32<8>(integrand);
    case 9: return pick_plus_f32<9>(integrand);
    case 10: return pick_plus_f32<10>(integrand);
    case 11: return pick_plus_f32<11>(integrand);
    case 12: return pick_plus_f32<12>(integrand);
    case 13: return pick_plus_f32<13>(integrand);
    case 14: return pick_plus_f32<14>(integrand);
    case 15: return pick_plus_f32<15>(integrand);
    case 16: return pick_plus_f32<16>(integrand);
    default: return nullptr;
  }
}

}  // namespace vf
