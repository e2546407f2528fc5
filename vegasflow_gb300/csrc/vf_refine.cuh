// The grid refinement of one dimension (vflow.py:135-211), shared by the
// VEGAS and VEGAS+ iteration-end kernels.
#pragma once
#include "vf_device.cuh"

namespace vf {

// Sum the 50 histogram columns of one dimension over `rows` partial rows into
// hsm[50] (and hist_out when given), by LANES x 50 threads of the block.
// `row_at(r)` returns the address of the dimension's first column in row r.
// Lane l takes rows l, l + LANES, ... with four independent accumulators (four
// loads in flight); the lanes are then added in order 0..LANES-1, so the
// result is fixed.  Ends with a barrier (every thread of the block calls it).
template <int LANES, typename RowAt>
__device__ inline void sum_hist_columns(RowAt row_at, int rows, double* hsm, double* hist_out) {
  __shared__ double part[LANES][VF_BINS];
  const int t = threadIdx.x;
  const int c = t % VF_BINS, l = t / VF_BINS;
  if (l < LANES) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int r = l;
    for (; r + 3 * LANES < rows; r += 4 * LANES) {
      s0 += row_at(r)[c];
      s1 += row_at(r + LANES)[c];
      s2 += row_at(r + 2 * LANES)[c];
      s3 += row_at(r + 3 * LANES)[c];
    }
    for (; r < rows; r += LANES) s0 += row_at(r)[c];
    part[l][c] = (s0 + s1) + (s2 + s3);
  }
  __syncthreads();
  if (t < VF_BINS) {
    double v = part[0][t];
    for (int i = 1; i < LANES; ++i) v += part[i][t];
    hsm[t] = v;
    if (hist_out) hist_out[t] = v;
  }
  __syncthreads();
}

// Sum of 50 values in NumPy's order for a contiguous float64 array of that
// length (np.sum: eight strided accumulators, a fixed tree, then the two
// remaining values), so the result is the oracle's bit for bit.  Called by
// all 32 lanes of one warp; the result is valid in lane 0.
__device__ inline double sum50_pairwise(const double* v) {
  const int j = threadIdx.x & 31;
  double r = 0.0;
  if (j < 8) {
    r = v[j];
    for (int i = 8; i < 48; i += 8) r += v[i + j];
  }
  r += __shfl_down_sync(0xffffffffu, r, 1);  // lanes 0, 2, 4, 6: r0+r1, r2+r3, ...
  r += __shfl_down_sync(0xffffffffu, r, 2);  // lanes 0, 4
  r += __shfl_down_sync(0xffffffffu, r, 4);  // lane 0
  r += v[48];
  r += v[49];
  return r;
}

// vflow.py:135-211 for one dimension, by one block of at least 64 threads.
// `h` is the dimension's 50-bin histogram in shared memory; `row` the
// dimension's 51 edges in global memory (read, then overwritten).
__device__ inline void refine_dimension(const double* h, double* row, double alpha, int* flags) {
  __shared__ double sub[VF_EDGES];
  __shared__ double sm[VF_BINS];
  __shared__ double wei[VF_BINS];
  __shared__ double sum_t;
  __shared__ int walk_bin[VF_BINS - 1];
  __shared__ double walk_weight[VF_BINS - 1];
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
  if (t < 32) {
    const double s = sum50_pairwise(sm);  // :162
    if (t == 0) sum_t = s;
  }
  __syncthreads();
  if (t < VF_BINS) {
    const double aux = (1.0 - sm[t] / sum_t) / (log(sum_t) - log(sm[t]));  // :163-164
    // :165; for the default alpha = 3/2, aux * sqrt(aux) (two correctly
    // rounded operations) in place of the general power
    wei[t] = alpha == 1.5 ? aux * sqrt(aux) : pow(aux, alpha);
  }
  __syncthreads();
  if (t < 32) {
    const double total = sum50_pairwise(wei);
    if (t == 0) {
      const double ave = total / VF_BINS;  // :166
      // :195-208, the while-loop state carried over the 49 outer steps.  Only
      // the additions are sequential: (n_bin, bin_weight) after each step is
      // recorded and the 49 new edges are computed in parallel below (cur and
      // prev follow from n_bin), with the same operations in the same order.
      // For a finite positive `ave`, bin_weight < ave is decided on the bit
      // patterns (IEEE order of a non-NaN double vs a positive one), which
      // keeps the comparisons off the float64 pipe.
      const bool int_cmp = isfinite(ave) && ave > 0.0;
      const long long ave_bits = __double_as_longlong(ave);
      double bin_weight = 0.0;
      int n_bin = -1;
      int overrun = 0;
      for (int k = 0; k < VF_BINS - 1; ++k) {
        while (int_cmp ? __double_as_longlong(bin_weight) < ave_bits : bin_weight < ave) {
          if (n_bin + 1 >= VF_BINS) {
            overrun = 1;
            break;
          }
          n_bin += 1;
          bin_weight += wei[n_bin];
        }
        bin_weight -= ave;
        walk_bin[k] = n_bin;
        walk_weight[k] = bin_weight;
      }
      if (overrun && flags) atomicOr(flags, VF_FLAG_REFINE_OVERRUN);
    }
  }
  __syncthreads();
  if (t < VF_BINS - 1) {
    const int n_bin = walk_bin[t];
    // cur = edge n_bin + 1 and prev = the cur before it; both start at 0 before
    // the first bin is entered (n_bin = -1 only if the weights are not finite)
    const double cur = n_bin >= 0 ? sub[n_bin + 1] : 0.0;
    const double prev = n_bin >= 1 ? sub[n_bin] : 0.0;
    const double w = wei[n_bin >= 0 ? n_bin : VF_BINS - 1];
    const double delta = (cur - prev) * walk_weight[t] / w;
    row[t + 1] = cur - delta;
  } else if (t == VF_BINS - 1) {
    row[0] = 0.0;
  } else if (t == VF_BINS) {
    row[VF_BINS] = 1.0;
  }
  __syncthreads();
}

}  // namespace vf
