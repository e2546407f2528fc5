// Ahead-of-time instantiations of the fp32 VEGAS map kernel (dimensions 1-16,
// 256 threads per block).
#include "vf_internal.h"
#include "vf_map_f32.cuh"

namespace vf {

const void* vegas_f32_map_kernel(int n_dim) {
  switch (n_dim) {
    case 1: return (const void*)vf_vegas_f32_map_kernel<1>;
    case 2: return (const void*)vf_vegas_f32_map_kernel<2>;
    case 3: return (const void*)vf_vegas_f32_map_kernel<3>;
    case 4: return (const void*)vf_vegas_f32_map_kernel<4>;
    case 5: return (const void*)vf_vegas_f32_map_kernel<5>;
    case 6: return (const void*)vf_vegas_f32_map_kernel<6>;
    case 7: return (const void*)vf_vegas_f32_map_kernel<7>;
    case 8: return (const void*)vf_vegas_f32_map_kernel<8>;
    case 9: return (const void*)vf_vegas_f32_map_kernel<9>;
    case 10: return (const void*)vf_vegas_f32_map_kernel<10>;
    case 11: return (const void*)vf_vegas_f32_map_kernel<11>;
    case 12: return (const void*)vf_vegas_f32_map_kernel<12>;
    case 13: return (const void*)vf_vegas_f32_map_kernel<13>;
    case 14: return (const void*)vf_vegas_f32_map_kernel<14>;
    case 15: return (const void*)vf_vegas_f32_map_kernel<15>;
    case 16: return (const void*)vf_vegas_f32_map_kernel<16>;
    default: return nullptr;
  }
}

}  // namespace vf
