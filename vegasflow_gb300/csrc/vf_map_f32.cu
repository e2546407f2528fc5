// Ahead-of-time instantiations of the fp32 VEGAS map kernel (dimensions 1-16;
// with and without bin-index output).
#include "vf_internal.h"
#include "vf_map_f32.cuh"

namespace vf {

namespace {

template <int D>
const void* pick_range(int n_dim, bool ind) {
  if constexpr (D > VF_MAX_DIM)
    return nullptr;
  else if (n_dim == D)
    return ind ? (const void*)vf_vegas_f32_map_kernel<D, true> : (const void*)vf_vegas_f32_map_kernel<D, false>;
  else
    return pick_range<D + 1>(n_dim, ind);
}

}  // namespace

const void* vegas_f32_map_kernel(int n_dim, bool ind) { return pick_range<1>(n_dim, ind); }

}  // namespace vf
