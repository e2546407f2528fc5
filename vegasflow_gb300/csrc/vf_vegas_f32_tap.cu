// Parity instantiations of the fp32 VEGAS Philox sampler (TAP = true: every
// event's bin indices written to ind_out), 1024 threads per block, dimensions 1-16, for
// the symmetric Gaussian (the benchmarked integrand) and the product integrand
// (whose table holds the point itself).  Tests reach them through vf_sample
// with ind_out as the only tap.
#include "vf_internal.h"
#include "vf_vegas_f32.cuh"

namespace vf {

template <int D>
static const void* pick_tap(int integrand) {
  switch (integrand) {
    case VF_INT_SYMGAUSS: return (const void*)vf_vegas_f32_kernel<D, VF_INT_SYMGAUSS, 1024, true>;
    case VF_INT_PROD: return (const void*)vf_vegas_f32_kernel<D, VF_INT_PROD, 1024, true>;
    default: return nullptr;
  }
}

const void* vegas_f32_tap_kernel(int n_dim, int integrand) {
  switch (n_dim) {
    case 1: return pick_tap<1>(integrand);
    case 2: return pick_tap<2>(integrand);
    case 3: return pick_tap<3>(integrand);
    case 4: return pick_tap<4>(integrand);
    case 5: return pick_tap<5>(integrand);
    case 6: return pick_tap<6>(integrand);
    case 7: return pick_tap<7>(integrand);
    case 8: return pick_tap<8>(integrand);
    case 9: return pick_tap<9>(integrand);
    case 10: return pick_tap<10>(integrand);
    case 11: return pick_tap<11>(integrand);
    case 12: return pick_tap<12>(integrand);
    case 13: return pick_tap<13>(integrand);
    case 14: return pick_tap<14>(integrand);
    case 15: return pick_tap<15>(integrand);
    case 16: return pick_tap<16>(integrand);
    default: return nullptr;
  }
}

}  // namespace vf
