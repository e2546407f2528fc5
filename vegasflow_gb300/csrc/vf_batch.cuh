// Batched VEGAS, the iteration end: per integral the sum of its tiles' partial
// rows, sigma, history, weighted average and chi2, and the refinement of every
// grid row (the sampler side is in vf_batch_sampler.cuh).
#pragma once
#include "vf_batch_sampler.cuh"
#include "vf_refine.cuh"

namespace vf {

// Batched iteration end: block b serves (item blk_item[b], role blk_role[b]);
// role d >= 0 sums histogram column d over the item's tiles and refines that
// grid row; role -1 sums res/res2, sigma, history and the weighted average of
// the item's slot, then advances the slot's counters.  Block 0 re-arms the
// sampler's work queue (the sampler launch has completed: stream order).
struct BatchEndArgs {
  const BatchItem* items;
  const int* blk_item;
  const int* blk_role;
  const long long* tile_row;
  const double* partials;
  double* grids;
  double* history;          // [slots][hist_cap][2]
  double* avg;              // [slots][5]
  int* iters;               // [slots] iterations in the current average (history index)
  unsigned int* calls;      // [slots] Philox call counters
  int* queue;               // the sampler's work counter, re-armed here
  int* flags;
  double* status;           // nullable [items][3]: mean, sigma, iterations (device address)
  double alpha;
  int hist_cap;
};

// Threads of an iteration-end block: 10 lanes per histogram bin, so that an
// integral of 512 tile rows costs each thread ~51 row loads in 4 independent
// chains (the rows were just written by the sampler and sit in L2).  Measured
// on the served stream: 24 us for such an integral with 10 lanes, 40 us with
// 5 (256 threads), 24 us with 20 (1024 threads, which made the 1,024-integral
// batch's ~10,000 small blocks run one per SM: +0.6 ms per iteration).
#define VF_BATCH_END_THREADS 512
#define VF_BATCH_END_LANES 10

__global__ void __launch_bounds__(VF_BATCH_END_THREADS) vf_batch_end_kernel(const BatchEndArgs a) {
  const int t = threadIdx.x;
  // re-arm the sampler's work queue (the sampler launch has completed: stream order)
  if (blockIdx.x == 0 && t == 0) *a.queue = 0;
  const int item = a.blk_item[blockIdx.x];
  const int role = a.blk_role[blockIdx.x];
  const BatchItem it = a.items[item];
  __shared__ double hsm[VF_BINS];
  __shared__ double red[2][VF_BATCH_END_THREADS / 32];
  if (role >= 0) {
    if (!it.train) return;
    const double* partials = a.partials + 2 + role * VF_BINS;
    const long long* rows = a.tile_row + it.tile0;
    sum_hist_columns<VF_BATCH_END_LANES>([=](int k) { return partials + rows[k]; }, it.n_tiles, hsm, nullptr);
    refine_dimension_f32(hsm, a.grids + it.grid_off + role * VF_EDGES, a.alpha, a.flags);
    return;
  }
  double s1 = 0.0, s2 = 0.0;
  for (int k = t; k < it.n_tiles; k += blockDim.x) {
    const double* row = a.partials + a.tile_row[it.tile0 + k];
    s1 += row[0];
    s2 += row[1];
  }
  // fixed order: lanes by a butterfly, then warps in order
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if ((t & 31) == 0) {
    red[0][t >> 5] = s1;
    red[1][t >> 5] = s2;
  }
  __syncthreads();
  if (t == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      red[0][0] += red[0][w];
      red[1][0] += red[1][w];
    }
  }
  __syncthreads();
  __shared__ double s_mean;
  __shared__ int s_hs;
  const int slot = it.slot;
  if (t == 0) {
    const int iter = a.iters[slot];
    const int hs = iter < a.hist_cap ? iter : a.hist_cap - 1;
    s_hs = hs;
    const double res = red[0][0], res2 = red[1][0];
    const double N = (double)it.n_events;
    const double err = __ddiv_rn(__dsub_rn(__dmul_rn(N, res2), __dmul_rn(res, res)), __dsub_rn(N, 1.0));
    const double sigma = sqrt(fmax(err, 0.0));
    double* h = a.history + ((long long)slot * a.hist_cap + hs) * 2;
    h[0] = res;
    h[1] = sigma;
    double* av = a.avg + 5LL * slot;
    const double wgt = 1.0 / __dmul_rn(sigma, sigma);
    av[0] = __dadd_rn(av[0], __dmul_rn(res, wgt));
    av[1] = __dadd_rn(av[1], wgt);
    const double mean = av[0] / av[1];
    av[2] = mean;
    av[3] = sqrt(1.0 / av[1]);
    s_mean = mean;
    if (!isfinite(res) && a.flags) atomicOr(a.flags, VF_FLAG_NONFINITE);
    a.iters[slot] = iter + 1;
    a.calls[slot] += 1u;
    if (a.status) {
      double* st = a.status + 3LL * item;
      st[0] = mean;
      st[1] = av[3];
      st[2] = (double)(iter + 1);
    }
  }
  __syncthreads();
  const double chi2 = block_chi2(a.history + (long long)slot * a.hist_cap * 2, 2, 1, s_hs + 1, s_mean);
  if (t == 0) a.avg[5LL * slot + 4] = s_hs > 0 ? chi2 / s_hs : 0.0;
}

}  // namespace vf
