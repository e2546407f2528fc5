// The float64 VEGAS+ sampler (and the fp32 one for injected uniforms and
// per-event taps): one warp per hypercube.  Kept apart from the iteration-end
// kernels so that NVRTC can compile it around a user integrand.
#pragma once
#include "vf_plus_args.cuh"

namespace vf {

template <typename Real, int DMAX, int INTEG>
__global__ void __launch_bounds__(VF_THREADS) vf_plus_kernel(const PlusArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int D = a.n_dim;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr bool evaluate = (INTEG != VF_INT_NONE);
  const bool fill_hist = evaluate && a.train;
  const int nb = D * VF_BINS;
  double* edges = reinterpret_cast<double*>(smem);
  Real* hist = reinterpret_cast<Real*>(smem + D * VF_EDGES * 8);
  for (int k = tid; k < D * VF_EDGES; k += blockDim.x) edges[k] = a.grid[k];
  if (fill_hist)
    for (int k = tid; k < nb; k += blockDim.x) hist[k] = (Real)0;
  __syncthreads();

  IntegrandConsts<Real, DMAX> kc;
  load_consts<DMAX>(kc, INTEG == VF_INT_USER ? VF_INT_NONE : INTEG, a.params, D);
  const bool limits = a.xmin != nullptr;
  const double inv_strat = 1.0 / (double)a.n_strat;
  int bad = 0;
  double blk1 = 0.0, blk2 = 0.0;  // this warp's contribution to the block row (lane 0)
  u32 cw2, cw3;
  plus_call_words(a, cw2, cw3);

  const int gwarp = blockIdx.x * (blockDim.x >> 5) + warp;
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  for (int h = gwarp; h < a.n_hcubes; h += nwarps) {
    // coordinates of hypercube h (last dimension fastest)
    int p[DMAX];
    {
      int rem = h;
#pragma unroll
      for (int d = DMAX - 1; d >= 0; --d)
        if (d < D) {
          p[d] = rem % a.n_strat;
          rem /= a.n_strat;
        }
    }
    const int nev = a.n_ev[h];
    const long long e0 = a.ev_start[h];
    double s1 = 0.0, s2 = 0.0;
    for (int j = lane; j < nev; j += 32) {
      const long long e = e0 + j;
      double u[DMAX];
      if (a.u_inj != nullptr) {
#pragma unroll
        for (int d = 0; d < DMAX; ++d)
          if (d < D) u[d] = a.u_inj[e * D + d];
      } else {
        // 53-bit uniforms through the TECH_CUT affine (both precisions: the
        // stratified map needs the full resolution of p + u)
#pragma unroll
        for (int q = 0; q < (DMAX + 1) / 2; ++q)
          if (2 * q < D) {
            u32 c0 = (u32)e, c1 = (u32)((u64)e >> 32), c2 = cw2 | (u32)q, c3 = cw3;
            philox4x32_10_rk(c0, c1, c2, c3, a.rk);
            u[2 * q] = tech_cut(u53(c0, c1));
            if (2 * q + 1 < DMAX) u[2 * q + 1] = tech_cut(u53(c2, c3));
          }
      }
      Real x[DMAX];
      int ind[DMAX];
      double w = 1.0;
#pragma unroll
      for (int d = 0; d < DMAX; ++d)
        if (d < D) {
          double xn;
          if constexpr (sizeof(Real) == 8) {
            // vflowplus.py:72: (p + u) * 50 / n_strat, three roundings
            xn = __ddiv_rn(__dmul_rn(__dadd_rn((double)p[d], u[d]), 50.0), (double)a.n_strat);
          } else {
            xn = ((double)p[d] + u[d]) * 50.0 * inv_strat;
          }
          int i = (int)xn;
          if (i < 0 || i > VF_BINS - 1) {
            bad = 1;
            i = i < 0 ? 0 : VF_BINS - 1;
          }
          const double lo = edges[d * VF_EDGES + i];
          const double dl = __dsub_rn(edges[d * VF_EDGES + i + 1], lo);
          const double aux = __dsub_rn(xn, floor(xn));
          x[d] = (Real)__dadd_rn(lo, __dmul_rn(dl, aux));
          const double fac = __dmul_rn(dl, 50.0);
          w = (d == 0) ? fac : __dmul_rn(w, fac);
          ind[d] = i;
        }
      w = __ddiv_rn(w, (double)nev);   // vflowplus.py:77
      w = __dmul_rn(w, a.xjac);        // monte_carlo.py:270
      if (limits) {
#pragma unroll
        for (int d = 0; d < DMAX; ++d)
          if (d < D) x[d] = (Real)__dadd_rn(a.xmin[d], __dmul_rn((double)x[d], a.xdelta[d]));
        w = __dmul_rn(w, a.xdeltajac);
      }
      if (evaluate) {
        double f;
#ifdef VF_JIT_USER
        if constexpr (INTEG == VF_INT_USER)
          f = (double)VF_USER_FN(x, D, (Real)w, a.params);
        else
#endif
          f = (double)eval_builtin<DMAX>(INTEG, x, D, kc);
        const double tmp = __dmul_rn(w, f);  // vflowplus.py:209
        const double tmp2 = __dmul_rn(tmp, tmp);
        s1 += tmp;
        s2 += tmp2;
        if (fill_hist) {
#pragma unroll
          for (int d = 0; d < DMAX; ++d)
            if (d < D) atomicAdd(hist + d * VF_BINS + ind[d], (Real)tmp2);
        }
      }
      if (a.ind_out) {
#pragma unroll
        for (int d = 0; d < DMAX; ++d)
          if (d < D) a.ind_out[e * D + d] = ind[d];
      }
      if (a.x_out) {
#pragma unroll
        for (int d = 0; d < DMAX; ++d)
          if (d < D) reinterpret_cast<Real*>(a.x_out)[e * D + d] = x[d];
      }
      if (a.w_out) reinterpret_cast<Real*>(a.w_out)[e] = (Real)w;
    }
    if (evaluate) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      }
      if (lane == 0) {
        a.ress[h] = s1;   // segment_sum, vflowplus.py:213-214
        a.ress2[h] = s2;
        blk1 += s1;
        blk2 += s2;
      }
    }
  }
  if (bad && a.flags) atomicOr(a.flags, VF_FLAG_INDEX_RANGE);
  if (!evaluate) return;
  __shared__ double red[2][VF_THREADS / 32];
  if (lane == 0) {
    red[0][warp] = blk1;
    red[1][warp] = blk2;
  }
  __syncthreads();
  double* row = a.partials + (long long)blockIdx.x * (2 + nb);
  if (tid == 0) {
    double b1 = 0.0, b2 = 0.0;
    for (int i = 0; i < VF_THREADS / 32; ++i) {
      b1 += red[0][i];
      b2 += red[1][i];
    }
    row[0] = b1;
    row[1] = b2;
  }
  if (fill_hist)
    for (int k = tid; k < nb; k += blockDim.x) row[2 + k] = (double)hist[k];
}

}  // namespace vf
