// The grid refinement of one dimension (vflow.py:135-211), shared by the
// VEGAS and VEGAS+ iteration-end kernels.
#pragma once
#include "vf_device.cuh"

namespace vf {

// vflow.py:135-211 for one dimension, by one block.  `h` is the dimension's
// 50-bin histogram in shared memory; `row` the dimension's 51 edges in global
// memory (read, then overwritten).
__device__ inline void refine_dimension(const double* h, double* row, double alpha, int* flags) {
  __shared__ double sub[VF_EDGES];
  __shared__ double sm[VF_BINS];
  __shared__ double wei[VF_BINS];
  __shared__ double sum_t;
  const int t = threadIdx.x;
  if (t < VF_EDGES) sub[t] = row[t];
  if (t < VF_BINS) {
    // res_padded[1:-1] + res_padded[2:] + res_padded[:-2], zero padding (:156-158)
    const double left = t > 0 ? h[t - 1] : 0.0;
    const double right = t < VF_BINS - 1 ? h[t + 1] : 0.0;
    const double v = (h[t] + right) + left;
    const double meaner = (t == 0 || t == VF_BINS - 1) ? 2.0 : 3.0;
    sm[t] = fmax(v / meaner, 1e-30);  // :159
  }
  __syncthreads();
  if (t == 0) {
    double s = 0.0;
    for (int i = 0; i < VF_BINS; ++i) s += sm[i];  // :162
    sum_t = s;
  }
  __syncthreads();
  if (t < VF_BINS) {
    const double aux = (1.0 - sm[t] / sum_t) / (log(sum_t) - log(sm[t]));  // :163-164
    wei[t] = pow(aux, alpha);                                               // :165
  }
  __syncthreads();
  if (t == 0) {
    double ave = 0.0;
    for (int i = 0; i < VF_BINS; ++i) ave += wei[i];
    ave = ave / VF_BINS;  // :166
    // :195-208, the while-loop state carried over the 49 outer steps
    double bin_weight = 0.0, cur = 0.0, prev = 0.0;
    int n_bin = -1;
    int overrun = 0;
    row[0] = 0.0;
    for (int k = 0; k < VF_BINS - 1; ++k) {
      while (bin_weight < ave) {
        if (n_bin + 1 >= VF_BINS) {
          overrun = 1;
          break;
        }
        n_bin += 1;
        bin_weight += wei[n_bin];
        prev = cur;
        cur = sub[n_bin + 1];
      }
      bin_weight -= ave;
      const double delta = (cur - prev) * bin_weight / wei[n_bin];
      row[k + 1] = cur - delta;
    }
    row[VF_BINS] = 1.0;
    if (overrun && flags) atomicOr(flags, VF_FLAG_REFINE_OVERRUN);
  }
  __syncthreads();
}

}  // namespace vf
