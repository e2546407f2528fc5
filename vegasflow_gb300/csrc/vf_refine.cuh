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
  if (count <= 32) {  // one warp holds every row (the other warps would add zeros): no block pass
    double c = 0.0;
    if (threadIdx.x < 32) {
      if ((int)threadIdx.x < count) {
        const double r = rows[(long long)threadIdx.x * stride], sg = rows[(long long)threadIdx.x * stride + sig_off];
        c = (r - mean) * (r - mean) / (sg * sg);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    return c;
  }
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
// histogram is scaled by a power of two 2^-e so its largest bin is about 1 (the
// refinement depends only on ratios and differences of logarithms), and the
// smoothed values are floored at the reference's absolute 1e-30 (vflow.py:159),
// i.e. at 1e-30 2^-e in scaled units, with the floor's logarithm carried
// separately (the scaled floor itself can leave float32's range: empty bins of
// a histogram whose largest bin is above ~1e8 would otherwise get a weight of
// 0, and flooring the scaled values at 1e-30 moved the edges of sparse
// histograms by up to 0.1), the smoothing, logarithms, damping and
// the rebinning run in float32 (a few hundred cycles instead of the float64
// pipe's ~15,000 on this part), and the new edges are made non-decreasing
// before they are stored as float64.  The rebinning walk of vflow.py:178-205
// (advance while the carried weight is below ave, subtract ave per new edge)
// is evaluated in parallel in its closed form: with P(i) the prefix sums of the
// weights, new edge k + 1 lies in the first bin n with P(n) >= (k + 1) ave, at
// the fraction (P(n) - (k + 1) ave) / wei[n] from its upper end -- a warp scan
// and one binary search per edge instead of one thread's ~100 dependent steps
// (which took ~4 us); the ordering of the edges is a prefix maximum.  The
// roundings differ from the sequential walk's by a few float32 ulps.
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
  __shared__ float prefix[VF_BINS];
  __shared__ float ave_sh;
  __shared__ float lsm[VF_BINS];        // log of the floored smoothed values (scaled)
  __shared__ float floor_sh, lfloor_sh;  // the floor 1e-30 in scaled units and its logarithm
  const int t = threadIdx.x;
  if (t < VF_EDGES) sub[t] = (float)row[t];
  if (t < 32) {  // the largest binary exponent among the 50 bins (integer max over the bit patterns)
    int e = -1022;
    for (int b = t; b < VF_BINS; b += 32) {
      const int ex = (int)((__double_as_longlong(h[b]) >> 52) & 0x7FF) - 1023;
      e = ex > e ? ex : e;
    }
    e = __reduce_max_sync(0xffffffffu, e);
    if (t == 0) {
      const int em = e > 1000 ? 1000 : e;
      emax = em;
      // 1e-30 2^-em: 0 or denormal when the histogram is large (only its
      // logarithm matters then), capped at 1e30 when it is tiny (every bin is
      // floored then, and the weights are uniform whatever the common value)
      float fl = ldexpf(1e-30f, -em);
      float lfl = -69.07755279f - (float)em * 0.69314718f;
      if (!(fl <= 1e30f)) {
        fl = 1e30f;
        lfl = 69.07755279f;
      }
      floor_sh = fl;
      lfloor_sh = lfl;
    }
  }
  __syncthreads();
  if (t < VF_BINS) hf[t] = (float)(h[t] * __longlong_as_double((long long)(1023 - emax) << 52));  // h 2^-emax
  __syncthreads();
  if (t < VF_BINS) {
    const float left = t > 0 ? hf[t - 1] : 0.0f;
    const float right = t < VF_BINS - 1 ? hf[t + 1] : 0.0f;
    const float v = (hf[t] + right) + left;
    const float meaner = (t == 0 || t == VF_BINS - 1) ? 2.0f : 3.0f;
    const float q = v / meaner;
    const bool floored = q < floor_sh || q == 0.0f;
    sm[t] = floored ? floor_sh : q;
    lsm[t] = floored ? lfloor_sh : logf(q);
  }
  __syncthreads();
  if (t < 32) {
    const float s = sum50_pairwise_f(sm);
    if (t == 0) sum_t = s;
  }
  __syncthreads();
  if (t < VF_BINS) {
    const float aux = (1.0f - sm[t] / sum_t) / (logf(sum_t) - lsm[t]);
    wei[t] = alpha == 1.5 ? aux * sqrtf(aux) : powf(aux, (float)alpha);
  }
  __syncthreads();
  if (t < 32) {
    const float total = sum50_pairwise_f(wei);
    // inclusive prefix sums P(i) of the weights: two bins per lane, a warp scan
    const int i0 = 2 * t, i1 = 2 * t + 1;
    const float a0 = i0 < VF_BINS ? wei[i0] : 0.0f;
    const float a1 = i1 < VF_BINS ? wei[i1] : 0.0f;
    float sc = a0 + a1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float u = __shfl_up_sync(0xffffffffu, sc, o);
      if (t >= o) sc += u;
    }
    float ex = __shfl_up_sync(0xffffffffu, sc, 1);
    if (t == 0) ex = 0.0f;
    const float p0 = ex + a0;
    if (i0 < VF_BINS) prefix[i0] = p0;
    if (i1 < VF_BINS) prefix[i1] = p0 + a1;
    if (t == 0) ave_sh = total / VF_BINS;
  }
  __syncthreads();
  if (t < VF_BINS - 1) {
    // new edge t + 1: the first bin whose prefix reaches (t + 1) ave
    const float target = (float)(t + 1) * ave_sh;
    int lo = 0, hi = VF_BINS;  // P(lo - 1) < target <= P(hi), as far as known
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (prefix[mid] < target)
        lo = mid + 1;
      else
        hi = mid;
    }
    int n_bin = lo;
    if (n_bin >= VF_BINS) {  // the walk would run past the last bin (rounding): the reference indexes out of range
      n_bin = VF_BINS - 1;
      if (flags) atomicOr(flags, VF_FLAG_REFINE_OVERRUN);
    }
    const float carried = prefix[n_bin] - target;
    const float cur = sub[n_bin + 1];
    const float prev = n_bin >= 1 ? sub[n_bin] : 0.0f;  // the walk starts from prev = 0 (vflow.py:197-199)
    edge[t + 1] = cur - (cur - prev) * carried / wei[n_bin];
  }
  __syncthreads();
  if (t < 32) {  // float32 rounding can swap two edges a few ulps apart: keep them ordered (a prefix maximum)
    const int k0 = 2 * t + 1, k1 = 2 * t + 2;  // edges 1..49
    const float e0 = k0 < VF_BINS ? fminf(edge[k0], 1.0f) : 0.0f;
    const float e1 = k1 < VF_BINS ? fminf(edge[k1], 1.0f) : 0.0f;
    float m = fmaxf(e0, e1);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float u = __shfl_up_sync(0xffffffffu, m, o);
      if (t >= o) m = fmaxf(m, u);
    }
    float before = __shfl_up_sync(0xffffffffu, m, 1);
    if (t == 0) before = 0.0f;
    const float m0 = fmaxf(before, e0);
    if (k0 < VF_BINS) row[k0] = (double)m0;
    if (k1 < VF_BINS) row[k1] = (double)fmaxf(m0, e1);
    if (t == 0) {
      row[0] = 0.0;
      row[VF_BINS] = 1.0;
    }
  }
  __syncthreads();
}

}  // namespace vf
