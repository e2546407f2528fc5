// Iteration-end work: reduce the per-block partial rows in a fixed order,
// sigma, the running 1/sigma^2-weighted average and chi^2, and the grid
// refinement (a cluster of 8 blocks per dimension, block 0 refining the row).
// Also the standalone refinement, the per-bin histogram utility and the
// reduction for torch-evaluated integrands.
#pragma once
#include "vf_device.cuh"
#include "vf_refine.cuh"

#include <cooperative_groups.h>

namespace vf {

struct IterEndArgs {
  const double* partials;  // [rows][W], W = 2 n_out + 50 D
  double* grid;            // [D][51], refined in place when train
  double* hist_out;        // nullable [D][50]: the iteration's arr_res2
  double* sums_out;        // nullable [2 n_out]: res, res2
  double* history;         // [iterations][2 n_out]: res[n_out], sigma[n_out]
  double* avg;             // [n_out][5]: sum res/s^2, sum 1/s^2, mean, sigma, chi2/dof
  int* flags;              // nullable
  double n_events;         // events of the iteration (the reference's n_events)
  double alpha;            // grid damping exponent
  int rows;
  int n_dim;
  int n_out;
  int train;               // 0 no refinement, 1 refine in float64, 2 refine in float32
  int iter;
  // nullable: the iteration index in device memory (read instead of `iter`,
  // then advanced, with the Philox call counter `call_dev`, for the next
  // iteration: a launch replayed from a CUDA graph); history has hist_cap rows
  int* iter_dev;
  unsigned int* call_dev;
  int hist_cap;
};

// The iteration-end kernel runs in clusters of VF_END_CLUSTER blocks: cluster
// d < D reduces dimension d's histogram columns, each block over 1/8 of the
// partial rows (the float64 additions spread over 8 SMs), and block 0 of the
// cluster adds the 8 block sums in rank order through distributed shared
// memory and refines the grid row.  The last cluster's block 0 does the
// integral sums.  Every sum has a fixed order, so the result does not depend
// on scheduling.
#define VF_END_CLUSTER 8
#define VF_END_THREADS 512
#define VF_END_LANES 10

__global__ void __cluster_dims__(VF_END_CLUSTER, 1, 1) __launch_bounds__(VF_END_THREADS)
vf_iteration_end_kernel(const IterEndArgs a) {
  namespace cg = cooperative_groups;
  const cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int group = blockIdx.x / VF_END_CLUSTER;
  const int t = threadIdx.x;
  const int D = a.n_dim;
  const int K = a.n_out;
  const long long W = 2 * K + VF_BINS * D;
  __shared__ double mine[VF_BINS];
  __shared__ double hsm[VF_BINS];
  const bool per_dim = a.train || a.hist_out != nullptr;
  if (per_dim && group < D) {
    const int d = group;
    const int lo = (int)((long long)a.rows * rank / VF_END_CLUSTER);
    const int hi = (int)((long long)a.rows * (rank + 1) / VF_END_CLUSTER);
    const double* col0 = a.partials + 2 * K + d * VF_BINS + lo * W;
    sum_hist_columns<VF_END_LANES>([=](int r) { return col0 + r * W; }, hi - lo, mine, nullptr);
    cluster.sync();
    if (rank == 0 && t < VF_BINS) {
      double v = mine[t];
      for (int r = 1; r < VF_END_CLUSTER; ++r) v += cluster.map_shared_rank(mine, r)[t];
      hsm[t] = v;
      if (a.hist_out) a.hist_out[d * VF_BINS + t] = v;
    }
    cluster.sync();  // the other blocks keep their shared memory until block 0 has read it
    if (rank == 0 && a.train == 1) refine_dimension(hsm, a.grid + d * VF_EDGES, a.alpha, a.flags);
    if (rank == 0 && a.train == 2) refine_dimension_f32(hsm, a.grid + d * VF_EDGES, a.alpha, a.flags);
    return;
  }
  if (rank != 0) return;
  const int it = a.iter_dev ? *a.iter_dev : a.iter;
  if (it < 0 || (a.iter_dev && it >= a.hist_cap)) {  // no history row left: report, change nothing
    if (t == 0 && a.flags) atomicOr(a.flags, VF_FLAG_HISTORY_FULL);
    return;
  }
  // ---- the sums, one output at a time: each thread's rows, then warp 0 adds
  // res and warp 1 res2 over the threads' partials in a fixed order (float64
  // additions cost an SM sub-partition 64 cycles each: two warps on two
  // sub-partitions beat a butterfly in every warp plus a serial pass)
  __shared__ double part[2][VF_END_THREADS];
  __shared__ double tot[2];
  __shared__ double mean_sh, sums_sh[2];
  const int lane = t & 31, warp = t >> 5;
  for (int j = 0; j < K; ++j) {
    double s1 = 0.0, s2 = 0.0;
    for (int r = t; r < a.rows; r += blockDim.x) {
      s1 += a.partials[(long long)r * W + j];
      s2 += a.partials[(long long)r * W + K + j];
    }
    part[0][t] = s1;
    part[1][t] = s2;
    __syncthreads();
    if (warp < 2) {
      double v = 0.0;
#pragma unroll 4
      for (int i = lane; i < (int)blockDim.x; i += 32) v += part[warp][i];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) tot[warp] = v;
    }
    __syncthreads();
    if (t == 0) {
      const double res = tot[0], res2 = tot[1];
      const double N = a.n_events;
      // vflow.py:437-438 (and plain.py:37-43, the same expression)
      const double err_tmp2 = __ddiv_rn(__dsub_rn(__dmul_rn(N, res2), __dmul_rn(res, res)), __dsub_rn(N, 1.0));
      const double sigma = sqrt(fmax(err_tmp2, 0.0));
      if (a.sums_out) {
        a.sums_out[j] = res;
        a.sums_out[K + j] = res2;
      }
      double* hrow = a.history + (long long)it * 2 * K;
      hrow[j] = res;
      hrow[K + j] = sigma;
      // monte_carlo.py:712-732, accumulated iteration by iteration
      double* av = a.avg + 5 * j;
      const double wgt = 1.0 / __dmul_rn(sigma, sigma);
      // history row 0 starts a new average: the buffer's previous contents are not read
      av[0] = it == 0 ? __dmul_rn(res, wgt) : __dadd_rn(av[0], __dmul_rn(res, wgt));
      av[1] = it == 0 ? wgt : __dadd_rn(av[1], wgt);
      sums_sh[0] = av[0];
      sums_sh[1] = av[1];
      if (!isfinite(res) || !isfinite(res2)) {
        if (a.flags) atomicOr(a.flags, VF_FLAG_NONFINITE);
      }
    }
    __syncthreads();
    // the mean and its sigma, two independent float64 chains on two warps
    if (t == 0) {
      const double mean = sums_sh[0] / sums_sh[1];
      a.avg[5 * j + 2] = mean;
      mean_sh = mean;
    } else if (t == 32) {
      a.avg[5 * j + 3] = sqrt(1.0 / sums_sh[1]);
    }
    __syncthreads();
    const double chi2 = block_chi2(a.history + j, 2 * K, K, it + 1, mean_sh);
    if (t == 0) a.avg[5 * j + 4] = it > 0 ? chi2 / it : 0.0;
  }
  if (t == 0 && a.iter_dev) {  // the next iteration's index and Philox call
    *a.iter_dev = it + 1;
    if (a.call_dev) *a.call_dev += 1u;
  }
}

// The reference's refine_grid(arr_res2): one block per dimension.
__global__ void __launch_bounds__(64) vf_refine_kernel(double* grid, const double* hist, double alpha,
                                                        int* flags) {
  __shared__ double hsm[VF_BINS];
  const int d = blockIdx.x;
  if (threadIdx.x < VF_BINS) hsm[threadIdx.x] = hist[d * VF_BINS + threadIdx.x];
  __syncthreads();
  refine_dimension(hsm, grid + d * VF_EDGES, alpha, flags);
}

// utils.py:17-44: out[b] = sum of input[e] with indices[e] == b.  `out` must be
// zeroed.  Shared-memory bins, then one float64 atomic per bin per block.
// The float64 uniforms u = (word + 1/2) / 2^32 that the fp32 samplers' integer
// maps stand for (word d of event e: Philox4x32-10 block q = d / 4 of counter
// (e, e >> 32, c2base | q, word3)), [n][n_dim] row-major.
__global__ void __launch_bounds__(256) vf_philox_uniforms_kernel(RoundKeys rk, unsigned int c2base,
                                                                 unsigned int word3, long long ev_offset,
                                                                 long long n, int n_dim, double* __restrict__ u) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    const unsigned long long ev = (unsigned long long)(ev_offset + e);
    for (int q = 0; 4 * q < n_dim; ++q) {
      unsigned int c0 = (unsigned int)ev, c1 = (unsigned int)(ev >> 32), c2 = c2base | (unsigned int)q, c3 = word3;
      philox4x32_10_rk(c0, c1, c2, c3, rk);
      const unsigned int w[4] = {c0, c1, c2, c3};
      for (int j = 0; j < 4 && 4 * q + j < n_dim; ++j)
        u[e * n_dim + 4 * q + j] = ((double)w[j] + 0.5) * 2.3283064365386962890625e-10;
    }
  }
}

__global__ void __launch_bounds__(256) vf_consume_kernel(const double* __restrict__ in,
                                                         const int* __restrict__ idx, long long n,
                                                         int size, double* out, int* flags) {
  extern __shared__ double bins[];
  for (int k = threadIdx.x; k < size; k += blockDim.x) bins[k] = 0.0;
  __syncthreads();
  int bad = 0;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const int b = idx[e];
    if (b < 0 || b >= size) {
      bad = 1;
      continue;
    }
    atomicAdd(&bins[b], in[e]);
  }
  if (bad && flags) atomicOr(flags, VF_FLAG_INDEX_RANGE);
  __syncthreads();
  for (int k = threadIdx.x; k < size; k += blockDim.x)
    if (bins[k] != 0.0) atomicAdd(&out[k], bins[k]);
}

// Partial rows from integrand values computed outside the sampler (torch
// callables): tmp = w f, tmp2 = tmp^2 per output; histogram of the main output.
struct ReduceArgs {
  const void* f;       // [n][n_out] (Real)
  const void* w;       // [n] (Real), the full weight
  const int* ind;      // [n][D]
  double* partials;    // [rows][W], W = 2 n_out + 50 D
  int* flags;
  long long n_events;
  int n_dim;
  int n_out;
  int main_dim;
  int train;
  int accumulate;
};

template <typename Real>
__global__ void __launch_bounds__(256) vf_reduce_events_kernel(const ReduceArgs a) {
  extern __shared__ double rsm[];  // [D*50] histogram, then [2][8][n_out] sums
  const int D = a.n_dim, K = a.n_out;
  const int nb = D * VF_BINS;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  double* hist = rsm;
  double* wred = rsm + nb;
  if (a.train)
    for (int k = t; k < nb; k += blockDim.x) hist[k] = 0.0;
  __syncthreads();
  const Real* f = reinterpret_cast<const Real*>(a.f);
  const Real* w = reinterpret_cast<const Real*>(a.w);
  double* row = a.partials + (long long)blockIdx.x * (2 * K + nb);
  for (int j = 0; j < K; ++j) {
    double s1 = 0.0, s2 = 0.0;
    for (long long e = (long long)blockIdx.x * blockDim.x + t; e < a.n_events;
         e += (long long)gridDim.x * blockDim.x) {
      // vflow.py:414-417: tmp = xjac * f (xjac reshaped to a column for vectorial f)
      const double tmp = (double)w[e] * (double)f[e * K + j];
      const double tmp2 = tmp * tmp;
      s1 += tmp;
      s2 += tmp2;
      if (a.train && j == a.main_dim)
        for (int d = 0; d < D; ++d) {
          const int b = a.ind[e * D + d];
          if (b >= 0 && b < VF_BINS) atomicAdd(&hist[d * VF_BINS + b], tmp2);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (lane == 0) {
      wred[warp] = s1;
      wred[8 + warp] = s2;
    }
    __syncthreads();
    if (t == 0) {
      double b1 = 0.0, b2 = 0.0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
        b1 += wred[i];
        b2 += wred[8 + i];
      }
      if (a.accumulate) {
        row[j] += b1;
        row[K + j] += b2;
      } else {
        row[j] = b1;
        row[K + j] = b2;
      }
    }
    __syncthreads();
  }
  if (a.train)
    for (int k = t; k < nb; k += blockDim.x) {
      if (a.accumulate)
        row[2 * K + k] += hist[k];
      else
        row[2 * K + k] = hist[k];
    }
}

}  // namespace vf
