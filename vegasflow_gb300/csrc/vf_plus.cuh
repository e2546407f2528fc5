// VEGAS+ (importance + adaptive stratified sampling) kernels.
//
// Events are laid out hypercube by hypercube: hypercube h owns the events
// [ev_start[h], ev_start[h] + n_ev[h]) of the iteration, with ev_start the
// exclusive prefix sum of n_ev (kept on the device, rebuilt by the
// reallocation step).  One warp processes one hypercube at a time, so the
// per-hypercube sums are warp reductions written by one lane (deterministic).
// Hypercube h has coordinates p_d = digit d of h in base n_strat, the last
// dimension fastest (the itertools.product order of vflowplus.py:126-128).
#pragma once
#include "vf_plus_args.cuh"
#include "vf_plus_sampler.cuh"
#include "vf_refine.cuh"
#include "vf_sample.cuh"

#include <cooperative_groups.h>

namespace vf {

// Torch-evaluated integrands: per-hypercube sums and histogram from f, w, ind.
struct PlusReduceArgs {
  const void* f;             // [n_events] (Real)
  const void* w;             // [n_events] (Real)
  const int* ind;            // [n_events][D]
  const int* n_ev;
  const long long* ev_start;
  double* ress;
  double* ress2;
  double* partials;
  int n_dim;
  int n_hcubes;
  int train;
};

template <typename Real>
__global__ void __launch_bounds__(VF_THREADS) vf_plus_reduce_kernel(const PlusReduceArgs a) {
  extern __shared__ double hsm[];
  const int D = a.n_dim, nb = D * VF_BINS;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (a.train)
    for (int k = tid; k < nb; k += blockDim.x) hsm[k] = 0.0;
  __syncthreads();
  const Real* f = reinterpret_cast<const Real*>(a.f);
  const Real* w = reinterpret_cast<const Real*>(a.w);
  const int gwarp = blockIdx.x * (blockDim.x >> 5) + warp;
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  for (int h = gwarp; h < a.n_hcubes; h += nwarps) {
    const int nev = a.n_ev[h];
    const long long e0 = a.ev_start[h];
    double s1 = 0.0, s2 = 0.0;
    for (int j = lane; j < nev; j += 32) {
      const long long e = e0 + j;
      const double tmp = (double)w[e] * (double)f[e];
      const double tmp2 = tmp * tmp;
      s1 += tmp;
      s2 += tmp2;
      if (a.train)
        for (int d = 0; d < D; ++d) {
          const int b = a.ind[e * D + d];
          if (b >= 0 && b < VF_BINS) atomicAdd(&hsm[d * VF_BINS + b], tmp2);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (lane == 0) {
      a.ress[h] = s1;
      a.ress2[h] = s2;
    }
  }
  __syncthreads();
  double* row = a.partials + (long long)blockIdx.x * (2 + nb);
  if (tid == 0) {
    row[0] = 0.0;
    row[1] = 0.0;
  }
  if (a.train)
    for (int k = tid; k < nb; k += blockDim.x) row[2 + k] = hsm[k];
}

// Iteration end of VEGAS+ (vflowplus.py:222-241): result and sigma from the
// per-hypercube sums, the adaptive reallocation (vflowplus.py:153-163) with the
// new prefix sum, and -- in the other blocks -- the grid refinement.
struct PlusEndArgs {
  const double* ress;
  const double* ress2;
  int* n_ev;                 // [H], rewritten when adaptive
  long long* ev_start;       // [H + 1], rewritten when adaptive
  double* arr_var;           // nullable [H] out: ress2 n_ev - ress^2
  const double* partials;    // histogram rows
  double* grid;
  double* hist_out;
  double* history;           // [iter][2]
  double* avg;               // [5]
  int* flags;
  double init_calls;         // N0, the constructor's n_events
  double alpha;
  double beta;
  int n_hcubes;
  int min_neval;
  int adaptive;
  int rows;
  int n_dim;
  int train;
  int iter;
  // nullable: the iteration index in device memory, read here (instead of
  // `iter`) and then advanced with the Philox call counter `call_dev` for the
  // next iteration (a launch replayed from a CUDA graph); history has hist_cap rows
  int* iter_dev;
  unsigned int* call_dev;
  int hist_cap;
};

// var^(beta/2), vflowplus.py:157.  For the default beta = 3/4 the power 3/8 is
// ((v^(1/2))^(1/2))^(1/2) cubed: three correctly rounded square roots and two
// products, about a third of the float64 instructions of pow (this part issues
// one float64 warp instruction per 64 cycles).  NaN for v < 0, as pow.
__device__ __forceinline__ double plus_damp(double v, double beta) {
  if (beta == 0.75) {
    const double r = sqrt(sqrt(sqrt(v)));
    return r * r * r;
  }
  return pow(v, beta / 2.0);
}

// The same in float32 (the fp32 form's reallocation, as the reference's float32
// mode computes it).  NaN for v < 0, as powf.
__device__ __forceinline__ float plus_damp_f32(float v, double beta) {
  if (beta == 0.75) {
    const float r = sqrtf(sqrtf(sqrtf(v)));
    return r * r * r;
  }
  return powf(v, (float)(beta / 2.0));
}

#define VF_PEND_CLUSTER 8
#define VF_PEND_THREADS 512
#define VF_PEND_MAXC 4  // hypercubes per thread: up to 8 x 512 x 4 = 16384

// The VEGAS+ iteration end, in clusters of 8 blocks.  Cluster d < D sums
// dimension d's histogram columns (each block 1/8 of the rows, combined in rank
// order through distributed shared memory) and refines the grid row.  The last
// cluster owns the hypercubes: each block a contiguous eighth, each thread a
// contiguous run of at most VF_PEND_MAXC; it forms var, the sums for res and
// sigma and the damped variances (fixed-order block and cluster reductions),
// block 0 records the iteration, and -- adaptive -- every thread turns its damped
// variances into new counts, followed by an exclusive prefix sum over threads,
// blocks (through distributed shared memory) and hypercubes into ev_start.
__global__ void __cluster_dims__(VF_PEND_CLUSTER, 1, 1) __launch_bounds__(VF_PEND_THREADS)
vf_plus_iteration_end_kernel(const PlusEndArgs a) {
  namespace cg = cooperative_groups;
  const cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int group = blockIdx.x / VF_PEND_CLUSTER;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int D = a.n_dim;
  const int H = a.n_hcubes;
  const long long W = 2 + VF_BINS * D;
  __shared__ double mine[VF_BINS];
  __shared__ double hsm[VF_BINS];
  if ((a.train || a.hist_out) && group < D) {
    const int d = group;
    const int lo = (int)((long long)a.rows * rank / VF_PEND_CLUSTER);
    const int hi = (int)((long long)a.rows * (rank + 1) / VF_PEND_CLUSTER);
    const double* col0 = a.partials + 2 + d * VF_BINS + lo * W;
    sum_hist_columns<VF_PEND_THREADS / VF_BINS>([=](int r) { return col0 + r * W; }, hi - lo, mine, nullptr);
    cluster.sync();
    if (rank == 0 && t < VF_BINS) {
      double v = mine[t];
      for (int r = 1; r < VF_PEND_CLUSTER; ++r) v += cluster.map_shared_rank(mine, r)[t];
      hsm[t] = v;
      if (a.hist_out) a.hist_out[d * VF_BINS + t] = v;
    }
    cluster.sync();
    if (rank == 0 && a.train == 1) refine_dimension(hsm, a.grid + d * VF_EDGES, a.alpha, a.flags);
    if (rank == 0 && a.train == 2) refine_dimension_f32(hsm, a.grid + d * VF_EDGES, a.alpha, a.flags);
    return;
  }

  // ---- the hypercubes of this block, a contiguous run per thread
  const int lo = (int)((long long)H * rank / VF_PEND_CLUSTER);
  const int hi = (int)((long long)H * (rank + 1) / VF_PEND_CLUSTER);
  const int C = (hi - lo + VF_PEND_THREADS - 1) / VF_PEND_THREADS;
  const int h0 = lo + t * C;
  // the fp32 form (float32 refinement): the variance stays float64 (it cancels),
  // its sigma term's division, the damped variance and the new counts are float32
  // -- the reference's float32-mode arithmetic -- which takes ~35 of the ~45
  // float64 instructions per hypercube off this cluster's critical path
  const bool f32 = a.train == 2;
  double dmp[VF_PEND_MAXC];
  double r1 = 0.0, r2 = 0.0, r3 = 0.0;
#pragma unroll
  for (int j = 0; j < VF_PEND_MAXC; ++j) {
    dmp[j] = 0.0;
    const int h = h0 + j;
    if (j < C && h < hi) {
      // vflowplus.py:216-217, 230-233
      const double nev = (double)a.n_ev[h];
      const double var = __dsub_rn(__dmul_rn(a.ress2[h], nev), __dmul_rn(a.ress[h], a.ress[h]));
      if (a.arr_var) a.arr_var[h] = var;
      r1 += a.ress[h];
      if (f32) {
        r2 += (double)((float)fmax(var, 0.0) / (float)(a.n_ev[h] - 1));
        if (a.adaptive) {
          dmp[j] = (double)plus_damp_f32((float)var, a.beta);
          r3 += dmp[j];
        }
      } else {
        r2 += fmax(var, 0.0) / (nev - 1.0);
        if (a.adaptive) {
          dmp[j] = plus_damp(var, a.beta);
          r3 += dmp[j];
        }
      }
    }
  }
  // block sums in a fixed order: the threads' partials to shared memory, then
  // warp k < 3 adds sum k (16 strided values per lane, then a butterfly).  Every
  // float64 addition costs its SM sub-partition 64 cycles, so three warps on
  // three sub-partitions (36 additions each) beat a butterfly in all 16 warps
  // (15 additions each, four warps per sub-partition) plus a serial pass.
  __shared__ double part[3][VF_PEND_THREADS];
  __shared__ double tot[3];
  part[0][t] = r1;
  part[1][t] = r2;
  part[2][t] = r3;
  __syncthreads();
  if (warp < 3) {
    double v = 0.0;
#pragma unroll 4
    for (int i = lane; i < VF_PEND_THREADS; i += 32) v += part[warp][i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) tot[warp] = v;
  }
  cluster.sync();
  __shared__ double all[3];  // the cluster's totals, added in rank order in every block
  __shared__ float s_scale;  // the fp32 form's count scale N0 / 2 / sum d
  __shared__ double s_mean;
  __shared__ int s_it, s_room;  // the iteration index; whether its history row exists
  if (t == 0) {
    double c1 = 0.0, c2 = 0.0, c3 = 0.0;
    for (int r = 0; r < VF_PEND_CLUSTER; ++r) {
      const double* tr = cluster.map_shared_rank(tot, r);
      c1 += tr[0];
      c2 += tr[1];
      c3 += tr[2];
    }
    all[0] = c1;
    all[1] = c2;
    all[2] = c3;
    if (f32 && a.adaptive) s_scale = (float)(a.init_calls / 2.0 / c3);
    if (rank == 0) {
      const int it = a.iter_dev ? *a.iter_dev : a.iter;
      s_it = it;
      s_room = it >= 0 && (!a.iter_dev || it < a.hist_cap);
      if (!s_room) {  // no history row left: report; the average is left as it was
        if (a.flags) atomicOr(a.flags, VF_FLAG_HISTORY_FULL);
      } else {
        const double res = c1;
        const double sigma = sqrt(c2);
        double* hrow = a.history + (long long)it * 2;
        hrow[0] = res;
        hrow[1] = sigma;
        const double wgt = 1.0 / __dmul_rn(sigma, sigma);
        // history row 0 starts a new average: the buffer's previous contents are not read
        a.avg[0] = it == 0 ? __dmul_rn(res, wgt) : __dadd_rn(a.avg[0], __dmul_rn(res, wgt));
        a.avg[1] = it == 0 ? wgt : __dadd_rn(a.avg[1], wgt);
        const double mean = a.avg[0] / a.avg[1];
        a.avg[2] = mean;
        a.avg[3] = sqrt(1.0 / a.avg[1]);
        s_mean = mean;
        if (!isfinite(res) && a.flags) atomicOr(a.flags, VF_FLAG_NONFINITE);
      }
    }
  }
  __syncthreads();
  if (rank == 0 && s_room) {
    const int it = s_it;
    const double chi2 = block_chi2(a.history, 2, 1, it + 1, s_mean);
    if (t == 0) {
      a.avg[4] = it > 0 ? chi2 / it : 0.0;
      if (a.iter_dev) {  // the next iteration's index and Philox call (the sampler has run: stream order)
        *a.iter_dev = it + 1;
        if (a.call_dev) *a.call_dev += 1u;
      }
    }
  }
  if (!a.adaptive) {
    cluster.sync();  // the other blocks' totals stay readable until every block has read them
    return;
  }

  // ---- reallocation, vflowplus.py:157-163: n_ev = int(max(min_neval, d N0 / 2 / sum d))
  const double sum_d = all[2];
  long long cnt[VF_PEND_MAXC];
  long long own = 0;
#pragma unroll
  for (int j = 0; j < VF_PEND_MAXC; ++j) {
    cnt[j] = 0;
    if (j < C && h0 + j < hi) {
      if (f32) {
        const float nn = fmaxf((float)a.min_neval, (float)dmp[j] * s_scale);  // one float32 product
        cnt[j] = (long long)(int)nn;
      } else {
        const double nn = fmax((double)a.min_neval, dmp[j] * a.init_calls / 2.0 / sum_d);
        cnt[j] = (long long)(int)nn;
      }
      own += cnt[j];
    }
  }
  // exclusive prefix of `own` over the block's threads (thread order = hypercube order)
  long long inc = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long v = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += v;
  }
  __shared__ long long wsum[VF_PEND_THREADS / 32];
  __shared__ long long btot;
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (t == 0) {
    long long acc = 0;
    for (int w = 0; w < VF_PEND_THREADS / 32; ++w) {
      const long long v = wsum[w];
      wsum[w] = acc;
      acc += v;
    }
    btot = acc;
  }
  cluster.sync();  // every block's total is ready
  __shared__ long long boff;
  if (t == 0) {
    long long off = 0, all_ev = 0;
    for (int r = 0; r < VF_PEND_CLUSTER; ++r) {
      const long long v = *cluster.map_shared_rank(&btot, r);
      if (r < rank) off += v;
      all_ev += v;
    }
    boff = off;
    if (rank == 0) a.ev_start[H] = all_ev;
  }
  __syncthreads();
  long long e = boff + wsum[warp] + inc - own;
#pragma unroll
  for (int j = 0; j < VF_PEND_MAXC; ++j) {
    const int h = h0 + j;
    if (j < C && h < hi) {
      a.n_ev[h] = (int)cnt[j];
      a.ev_start[h] = e;
      e += cnt[j];
    }
  }
  cluster.sync();  // the distributed reads above are done before any block exits
}

}  // namespace vf
