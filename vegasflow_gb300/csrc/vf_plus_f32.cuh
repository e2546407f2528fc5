// The fp32 VEGAS+ sampler: hypercube-stratified importance sampling
// (vflowplus.py:46-80, 187-220) with float32 arithmetic and an exact integer
// stratified map, for built-in integrands and in-kernel Philox uniforms.
//
// One warp per hypercube (events [ev_start[h], ev_start[h] + n_ev[h]), lanes
// strided), as the float64 kernel.  Per event and dimension one 32-bit Philox
// word w gives u = (w + 1/2) / 2^32, and the reference's stratified coordinate
// xn = (p + u) 50 / n_strat is taken exactly in integers:
//     Q = 50 (p 2^32 + w) + 25 = 50 (p + u) 2^32,   A = Q >> 32,  R = Q mod 2^32
//     bin = A div n_strat,  fraction = ((A mod n_strat) + R / 2^32) / n_strat
// (A < 50 n_strat, so the division is done in float32 and corrected by one
// step).  Then x = c0 + c1 m through the per-bin table {c0, c1} (float32,
// rounded once from float64, integration limits folded), the weight
// prod(c1) 50^D xjac / n_ev, the integrand in float32, per-hypercube sums with
// TwoSum-compensated float32 warp reductions written as float64, and the
// (w f)^2 histogram in shared tables, VF_PLUS_HIST_COPIES per warp.
#pragma once
#include "vf_plus_args.cuh"

namespace vf {

// Histogram copies per warp, one per group of 32 / VF_PLUS_HIST_COPIES lanes.  The
// lanes of a warp sample one hypercube, whose events fall in the same ~50 / n_strat
// bins of every dimension, so one table per warp makes the float atomics (compare-
// and-swap loops) of a warp instruction collide on a handful of addresses.
#define VF_PLUS_HIST_COPIES 4

__host__ __device__ inline int plus_f32_smem_bytes(int D, int train, int threads = VF_THREADS) {
  return D * VF_BINS * 8 + (train ? (threads / 32) * VF_PLUS_HIST_COPIES * D * VF_BINS * 4 : 0);
}

// TAP: the parity instantiation, which also writes every event's bin indices
// (a.ind_out, [n_events][D] int32) and point (a.x_out, float32, when not NULL)
// in event order; the kernels of the hot path are TAP = false.
template <int D, int INTEG, bool TAP = false>
__global__ void __launch_bounds__(VF_THREADS, D <= 8 ? 4 : 2) vf_plus_f32_kernel(const PlusArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NB = D * VF_BINS;
  float2* cells = reinterpret_cast<float2*>(smem);
  float* hist = reinterpret_cast<float*>(smem + NB * 8);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool train = a.train != 0;
  const bool limits = a.xmin != nullptr;
  for (int k = tid; k < NB; k += blockDim.x) {
    const int d = k / VF_BINS, b = k - d * VF_BINS;
    const double lo = a.grid[d * VF_EDGES + b];
    const double dl = a.grid[d * VF_EDGES + b + 1] - lo;
    double c0 = lo - dl, c1 = dl;
    if (limits) {
      c0 = __fma_rn(c0, a.xdelta[d], a.xmin[d]);
      c1 = c1 * a.xdelta[d];
    }
    cells[k] = make_float2((float)c0, (float)c1);
  }
  constexpr int NCOPIES = (VF_THREADS / 32) * VF_PLUS_HIST_COPIES;
  if (train)
    for (int k = tid; k < NCOPIES * NB; k += blockDim.x) hist[k] = 0.0f;
  __shared__ float s_wscale;
  if (tid == 0) {
    double ws = a.xjac;  // 1 / n_hcubes (vflowplus.py:144-146)
    for (int d = 0; d < D; ++d) ws *= 50.0;
    s_wscale = (float)ws;
  }
  __syncthreads();
  const float wscale = s_wscale;
  IntegrandConsts<float, D> kc;
  load_consts<D>(kc, INTEG == VF_INT_USER ? VF_INT_NONE : INTEG, a.params, D);
  float* my_hist = hist + (warp * VF_PLUS_HIST_COPIES + lane / (32 / VF_PLUS_HIST_COPIES)) * NB;
  u32 cw2, cw3;
  plus_call_words(a, cw2, cw3);
  const u32 ns = (u32)a.n_strat;
  const float inv_ns = 1.0f / (float)ns;
  double blk1 = 0.0, blk2 = 0.0;

  const int gwarp = blockIdx.x * (VF_THREADS / 32) + warp;
  const int nwarps = gridDim.x * (VF_THREADS / 32);
  for (int h = gwarp; h < a.n_hcubes; h += nwarps) {
    u32 p[D];  // hypercube coordinates, last dimension fastest (vflowplus.py:126-128)
    {
      u32 rem = (u32)h;
#pragma unroll
      for (int d = D - 1; d >= 0; --d) {
        p[d] = rem % ns;
        rem /= ns;
      }
    }
    const int nev = a.n_ev[h];
    const long long e0 = a.ev_start[h];
    const float wh = wscale / (float)nev;  // vflowplus.py:77
    F2 s1 = {0.0f, 0.0f}, s2 = {0.0f, 0.0f};
    for (int j = lane; j < nev; j += 32) {
      const u64 e = (u64)(e0 + j);
      float x[D];
      int bins[D];
      float wf = 1.0f;
#pragma unroll
      for (int q = 0; q < (D + 3) / 4; ++q) {
        u32 c0 = (u32)e, c1 = (u32)(e >> 32), c2 = cw2 | (u32)q, c3 = cw3;
        philox4x32_10_rk(c0, c1, c2, c3, a.rk);
        const u32 wq[4] = {c0, c1, c2, c3};
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const int d = 4 * q + jj;
          if (d < D) {
            const u64 Q = (((u64)p[d] << 32) | wq[jj]) * 50ull + 25ull;
            const u32 A = (u32)(Q >> 32), R = (u32)Q;
            u32 i = (u32)((float)A * inv_ns);  // A div n_strat, corrected below
            if (i * ns > A) --i;
            if ((i + 1) * ns <= A) ++i;
            const u32 r = A - i * ns;
            // m = 1 + fraction: (r + R 2^-32) / n_strat, two fused multiply-adds
            float m = fmaf(fmaf((float)R, 2.3283064e-10f, (float)r), inv_ns, 1.0f);
            m = fminf(m, 1.99999988f);  // keep the fraction below 1 after rounding
            const float2 c = cells[d * VF_BINS + i];
            x[d] = fmaf(c.y, m, c.x);
            wf = (d == 0) ? c.y : wf * c.y;
            bins[d] = d * VF_BINS + (int)i;
          }
        }
      }
      if constexpr (TAP) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
          a.ind_out[e * D + d] = bins[d] - d * VF_BINS;
          if (a.x_out) static_cast<float*>(a.x_out)[e * D + d] = x[d];
        }
      }
      float f;
#ifdef VF_JIT_USER
      if constexpr (INTEG == VF_INT_USER)
        f = (float)VF_USER_FN(x, D, wf * wh, a.params);
      else
#endif
        f = eval_builtin<D>(INTEG, x, D, kc);
      const float v = wf * wh * f;  // vflowplus.py:209
      const float v2 = v * v;
      two_sum_add(s1, v);
      two_sum_add(s2, v2);
      if (train) {
#pragma unroll
        for (int d = 0; d < D; ++d) atomicAdd(my_hist + bins[d], v2);
      }
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if (lane == 0) {
      const double r1 = (double)s1.s + (double)s1.c, r2 = (double)s2.s + (double)s2.c;
      a.ress[h] = r1;  // segment_sum, vflowplus.py:213-214
      a.ress2[h] = r2;
      blk1 += r1;
      blk2 += r2;
    }
  }
  __shared__ double red[2][VF_THREADS / 32];
  if (lane == 0) {
    red[0][warp] = blk1;
    red[1][warp] = blk2;
  }
  __syncthreads();
  double* row = a.partials + (long long)blockIdx.x * (2 + NB);
  if (tid == 0) {
    double b1 = 0.0, b2 = 0.0;
    for (int i = 0; i < VF_THREADS / 32; ++i) {
      b1 += red[0][i];
      b2 += red[1][i];
    }
    row[0] = b1;
    row[1] = b2;
  }
  if (train)
    for (int k = tid; k < NB; k += blockDim.x) {
      float hf = 0.0f;
      for (int c = 0; c < NCOPIES; ++c) hf += hist[c * NB + k];
      row[2 + k] = (double)hf;
    }
}

}  // namespace vf
