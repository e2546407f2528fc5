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

// chi^2 of `count` history rows against `mean`: sum over rows i of
// (r_i - mean)^2 / sigma_i^2, r_i = rows[i stride], sigma_i = rows[i stride +
// sig_off].  Rows are spread over the block's threads, then added lane by lane
// and warp by warp (a fixed order); every thread of the block calls it, the
// total is valid in thread 0.  (Each row costs a float64 division, ~1,000
// cycles on this part: one thread walking a long history was the iteration
// end's slowest step.)
__device__ inline double block_chi2(const double* rows, long long stride, int sig_off, int count, double mean) {
  __shared__ double part[32];
  double c = 0.0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) {
    const double r = rows[(long long)i * stride], sg = rows[(long long)i * stride + sig_off];
    c += (r - mean) * (r - mean) / (sg * sg);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
  __syncthreads();
  double total = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) total += part[w];
  __syncthreads();
  return total;
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

// The same refinement in float32 arithmetic -- the reference's float32 mode
// (configflow.py float switch) -- for the fp32 sampler's grids: the float64
// histogram is scaled by a power of two so its largest bin is about 1 (the
// refinement depends only on ratios, apart from the 1e-30 floor, which then
// applies relative to the largest bin), the smoothing, logarithms, damping and
// the rebinning walk run in float32 (a few hundred cycles instead of the
// float64 pipe's ~15,000 on this part), and the new edges are made
// non-decreasing before they are stored as float64.
__device__ inline float sum50_pairwise_f(const float* v) {
  const int j = threadIdx.x & 31;
  float r = 0.0f;
  if (j < 8) {
    r = v[j];
    for (int i = 8; i < 48; i += 8) r += v[i + j];
  }
  r += __shfl_down_sync(0xffffffffu, r, 1);
  r += __shfl_down_sync(0xffffffffu, r, 2);
  r += __shfl_down_sync(0xffffffffu, r, 4);
  r += v[48];
  r += v[49];
  return r;
}

__device__ inline void refine_dimension_f32(const double* h, double* row, double alpha, int* flags) {
  __shared__ float sub[VF_EDGES];
  __shared__ float hf[VF_BINS];
  __shared__ float sm[VF_BINS];
  __shared__ float wei[VF_BINS];
  __shared__ float edge[VF_EDGES];
  __shared__ float sum_t;
  __shared__ int emax;
  __shared__ int walk_bin[VF_BINS - 1];
  __shared__ float walk_weight[VF_BINS - 1];
  const int t = threadIdx.x;
  if (t < VF_EDGES) sub[t] = (float)row[t];
  if (t < 32) {  // the largest binary exponent among the 50 bins (integer max over the bit patterns)
    int e = -1022;
    for (int b = t; b < VF_BINS; b += 32) {
      const int ex = (int)((__double_as_longlong(h[b]) >> 52) & 0x7FF) - 1023;
      e = ex > e ? ex : e;
    }
    e = __reduce_max_sync(0xffffffffu, e);
    if (t == 0) emax = e > 1000 ? 1000 : e;
  }
  __syncthreads();
  if (t < VF_BINS) hf[t] = (float)(h[t] * __longlong_as_double((long long)(1023 - emax) << 52));  // h 2^-emax
  __syncthreads();
  if (t < VF_BINS) {
    const float left = t > 0 ? hf[t - 1] : 0.0f;
    const float right = t < VF_BINS - 1 ? hf[t + 1] : 0.0f;
    const float v = (hf[t] + right) + left;
    const float meaner = (t == 0 || t == VF_BINS - 1) ? 2.0f : 3.0f;
    sm[t] = fmaxf(v / meaner, 1e-30f);
  }
  __syncthreads();
  if (t < 32) {
    const float s = sum50_pairwise_f(sm);
    if (t == 0) sum_t = s;
  }
  __syncthreads();
  if (t < VF_BINS) {
    const float aux = (1.0f - sm[t] / sum_t) / (logf(sum_t) - logf(sm[t]));
    wei[t] = alpha == 1.5 ? aux * sqrtf(aux) : powf(aux, (float)alpha);
  }
  __syncthreads();
  if (t < 32) {
    const float total = sum50_pairwise_f(wei);
    if (t == 0) {
      const float ave = total / VF_BINS;
      float bin_weight = 0.0f;
      int n_bin = -1;
      int overrun = 0;
      for (int k = 0; k < VF_BINS - 1; ++k) {
        while (bin_weight < ave) {
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
    const float cur = n_bin >= 0 ? sub[n_bin + 1] : 0.0f;
    const float prev = n_bin >= 1 ? sub[n_bin] : 0.0f;
    const float w = wei[n_bin >= 0 ? n_bin : VF_BINS - 1];
    edge[t + 1] = cur - (cur - prev) * walk_weight[t] / w;
  }
  __syncthreads();
  if (t == 0) {  // float32 rounding can swap two edges a few ulps apart: keep them ordered
    float lo = 0.0f;
    row[0] = 0.0;
    for (int k = 1; k < VF_BINS; ++k) {
      lo = fmaxf(lo, fminf(edge[k], 1.0f));
      row[k] = (double)lo;
    }
    row[VF_BINS] = 1.0;
  }
  __syncthreads();
}

}  // namespace vf
