// The fused VEGAS / plain-MC sampler kernel.
//
// One thread per event in a grid-stride loop over a persistent grid (one
// partial row per block).  Per event: uniforms (in-kernel Philox, or injected
// from HBM), the importance map through the grid held in shared memory, the
// Jacobian weight, the integrand, and the accumulation of sum(w f), sum((w f)^2)
// and the per-bin histogram of (w f)^2.  Each block writes (or adds) one
// partial row  [res[0..n_out), res2[0..n_out), hist[D][50]]  in float64; the
// iteration-end kernel sums the rows in a fixed order.
//
//   Real = double : the reference's float64 arithmetic, operation by operation
//                   (bit-exact bin indices, points and weights).
//   Real = float  : the fused fp32 form.  Integer-domain map on one Philox word
//                   per dimension, fp32 evaluation, TwoSum-compensated per-thread
//                   and per-block sums, float64 from the block partial onward.
#pragma once
#include "vf_device.cuh"

#ifndef VF_THREADS
#define VF_THREADS 256
#endif

namespace vf {

struct SampleArgs {
  const double* grid;       // [D][51] bin edges (float64)
  const double* xmin;       // nullable [D] integration limits
  const double* xdelta;     // nullable [D]
  const double* u_inj;      // nullable [n_events][D] injected post-affine uniforms
  const double* params;     // integrand parameters
  double* partials;         // [rows][W], W = 2 + 50 D
  int* ind_out;             // nullable [n_events][D]
  void* x_out;              // nullable [n_events][D] (Real)
  void* w_out;              // nullable [n_events] (Real)
  void* f_out;              // nullable [n_events] (Real)
  int* flags;               // nullable error flags (VF_FLAG_*)
  long long n_events;       // events in this launch
  long long ev_offset;      // global index of the first event (Philox counter)
  double xjac;              // 1 / events per iteration (the reference's xjac)
  double xdeltajac;         // prod(xdelta), 1 without limits
  unsigned long long seed;  // Philox key
  unsigned int call_ctr;    // sampler call counter (one per iteration)
  int n_dim;
  int alg;                  // 0 = VEGAS importance map, 1 = plain MC
  int train;                // fill the histogram
  int accumulate;           // 0: store rows, 1: add to rows
  int hist_copies;          // generic kernel: 1 = one block histogram, >1 = per-warp copies;
                            // fp32 VEGAS kernel: copies per warp (1, 2, 4)
  RoundKeys rk;             // Philox round keys (seed + r W, r = 0..9), host-computed
  unsigned int ctr2[8];     // Philox counter word 2 of 4-word block q: (call << 4) | q;
                            // float64 uses ceil(D/2) <= 8 blocks, fp32 ceil(D/4) <= 4
  unsigned int ctr3;        // Philox counter word 3: call >> 28
  // nullable: the call counter in device memory, read by the kernel instead of
  // ctr2/ctr3 (a launch replayed from a CUDA graph, where the counter advances
  // on the device)
  const unsigned int* call_dev;
  // fp32 VEGAS kernel with injected uniforms: 0 = plain loads; 1|2|3 = tiles of
  // THREADS events brought into shared memory by TMA through `tmap`, with the
  // 32|64|128-byte swizzle (row bytes 8 D = 32|64|128)
  int tma_swizzle;
  int rows_total;           // partial rows the caller reduces; rows >= gridDim.x are cleared
  // CUtensorMap of u_inj as a [n_events][D] float64 tensor, box [THREADS][D]
  alignas(64) unsigned long long tmap[16];
};

// Philox counter words 2 (block 0; block q adds q) and 3 of a launch.
struct CallWords {
  u32 c2base, c3;
};
__device__ __forceinline__ CallWords call_words(const SampleArgs& a) {
  if (a.call_dev) {
    const u32 call = *a.call_dev;
    return {call << 4, call >> 28};
  }
  return {a.ctr2[0], a.ctr3};
}

// The 4 words of block q of event ev, with the host-computed keys.
__device__ __forceinline__ void philox_words(u64 ev, const SampleArgs& a, const CallWords& cw, int q, u32 w[4]) {
  u32 c0 = (u32)ev, c1 = (u32)(ev >> 32), c2 = cw.c2base | (u32)q, c3 = cw.c3;
  philox4x32_10_rk(c0, c1, c2, c3, a.rk);
  w[0] = c0;
  w[1] = c1;
  w[2] = c2;
  w[3] = c3;
}

template <typename Real>
struct GridSmemBytes;
template <>
struct GridSmemBytes<double> {
  static __host__ __device__ int bytes(int D) { return D * VF_EDGES * 8; }
};
template <>
struct GridSmemBytes<float> {
  static __host__ __device__ int bytes(int D) { return D * VF_BINS * 8; }
};

__host__ __device__ inline int sample_smem_bytes(int real_size, int D, int hist_copies, int train) {
  const int grid = real_size == 8 ? D * VF_EDGES * 8 : D * VF_BINS * 8;
  const int hist = train ? hist_copies * D * VF_BINS * real_size : 0;
  const int lim = 2 * VF_MAX_DIM * 8;
  return grid + hist + lim;
}

// ----- the integrand call ----------------------------------------------------
// VF_USER_FN names the user's device function when NVRTC compiles this header
// together with the user's source (VF_JIT_USER defined): it is declared before
// this header as  vf_real f(const vf_real* x, int n_dim, vf_real weight,
// const double* params)  with vf_real the sampler's precision.
template <typename Real, int DMAX, int INTEG>
__device__ __forceinline__ Real call_integrand(const Real* x, int D, Real w,
                                               const IntegrandConsts<Real, DMAX>& k,
                                               const double* __restrict__ params) {
#ifdef VF_JIT_USER
  if constexpr (INTEG == VF_INT_USER) return (Real)VF_USER_FN(x, D, w, params);
#endif
  return eval_builtin<DMAX>(INTEG, x, D, k);
}

// ----- block reductions --------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ F2 warp_sum(F2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    F2 t;
    t.s = __shfl_xor_sync(0xffffffffu, v.s, o);
    t.c = __shfl_xor_sync(0xffffffffu, v.c, o);
    v = two_sum_merge(v, t);
  }
  return v;
}

// ----- the kernel --------------------------------------------------------------
template <typename Real, int DMAX, int INTEG>
__global__ void __launch_bounds__(VF_THREADS)
vf_sample_kernel(const SampleArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int D = a.n_dim;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const bool vegas = (a.alg == 0);
  const bool evaluate = (INTEG != VF_INT_NONE);
  const bool fill_hist = evaluate && vegas && a.train;
  const bool limits = (a.xmin != nullptr);
  const int nb = D * VF_BINS;
  const CallWords cw = call_words(a);

  // shared-memory carve-up
  unsigned char* p = smem;
  double* edges = reinterpret_cast<double*>(p);  // fp64: [D][51]
  float2* cells = reinterpret_cast<float2*>(p);  // fp32: [D][50] {lo, delta}
  p += GridSmemBytes<Real>::bytes(D);
  Real* hist = reinterpret_cast<Real*>(p);
  p += fill_hist ? a.hist_copies * nb * (int)sizeof(Real) : 0;
  Real* lim = reinterpret_cast<Real*>(p);  // [2][VF_MAX_DIM] xmin, xdelta

  // the grid exists (and is read) only for the VEGAS map; plain MC passes NULL
  if constexpr (sizeof(Real) == 8) {
    if (vegas)
      for (int k = tid; k < D * VF_EDGES; k += blockDim.x) edges[k] = a.grid[k];
  } else if (vegas) {
    for (int k = tid; k < nb; k += blockDim.x) {
      const int d = k / VF_BINS, b = k - d * VF_BINS;
      const double lo = a.grid[d * VF_EDGES + b];
      const double hi = a.grid[d * VF_EDGES + b + 1];
      cells[k] = make_float2((float)lo, (float)(hi - lo));
    }
  }
  if (fill_hist)
    for (int k = tid; k < a.hist_copies * nb; k += blockDim.x) hist[k] = (Real)0;
  if (limits)
    for (int k = tid; k < D; k += blockDim.x) {
      lim[k] = (Real)a.xmin[k];
      lim[VF_MAX_DIM + k] = (Real)a.xdelta[k];
    }
  __syncthreads();

  IntegrandConsts<Real, DMAX> kc;
  load_consts<DMAX>(kc, INTEG == VF_INT_USER ? VF_INT_NONE : INTEG, a.params, D);
  Real* my_hist = hist + (warp % a.hist_copies) * nb;
  const double xjac = a.xjac;
  const double xdeltajac = a.xdeltajac;
  // float64 factor of the fp32 form's weight: 50^D (VEGAS Jacobian constant) * xjac * prod(xdelta)
  const double wscale = (sizeof(Real) == 8) ? 1.0 : (vegas ? pow(50.0, (double)D) : 1.0) * xjac * xdeltajac;
  const float wscale_f = (float)wscale;

  double acc1 = 0.0, acc2 = 0.0;  // fp64 accumulators
  F2 s1 = {0.0f, 0.0f}, s2 = {0.0f, 0.0f};  // fp32 compensated accumulators
  int bad = 0;

  const long long n = a.n_events;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + tid; e < n; e += stride) {
    const u64 ev = (u64)(a.ev_offset + e);
    Real x[DMAX];
    int ind[DMAX];
    Real w;

    if constexpr (sizeof(Real) == 8) {
      // ---------------- float64: the reference's operations ----------------
      double u[DMAX];
      if (a.u_inj != nullptr) {
        const double* up = a.u_inj + e * D;
#pragma unroll
        for (int d = 0; d < DMAX; ++d)
          if (d < D) u[d] = up[d];
      } else {
#pragma unroll
        for (int q = 0; q < (DMAX + 1) / 2; ++q)
          if (2 * q < D) {
            u32 wd[4];
            philox_words(ev, a, cw, q, wd);
            u[2 * q] = tech_cut(u53(wd[0], wd[1]));
            if (2 * q + 1 < DMAX) u[2 * q + 1] = tech_cut(u53(wd[2], wd[3]));
          }
      }
      double wd_ = 1.0;
      if (vegas) {
#pragma unroll
        for (int d = 0; d < DMAX; ++d)
          if (d < D) {
            const double xn = __dmul_rn(50.0, __dsub_rn(1.0, u[d]));  // vflow.py:117
            int i = (int)xn;                                           // vflow.py:67
            if (i < 0 || i > VF_BINS - 1) {
              bad = 1;
              i = i < 0 ? 0 : VF_BINS - 1;
            }
            const double lo = edges[d * VF_EDGES + i];
            const double dl = __dsub_rn(edges[d * VF_EDGES + i + 1], lo);  // :73
            const double aux = __dsub_rn(xn, floor(xn));                    // :75
            x[d] = (Real)__dadd_rn(lo, __dmul_rn(dl, aux));                 // :76
            const double fac = __dmul_rn(dl, 50.0);                         // :78
            wd_ = (d == 0) ? fac : __dmul_rn(wd_, fac);
            ind[d] = i;
          }
        wd_ = __dmul_rn(wd_, xjac);  // monte_carlo.py:270
      } else {
#pragma unroll
        for (int d = 0; d < DMAX; ++d)
          if (d < D) x[d] = (Real)u[d];
        wd_ = xjac;  // plain: 1.0 * xjac
      }
      if (limits) {  // monte_carlo.py:271-274
#pragma unroll
        for (int d = 0; d < DMAX; ++d)
          if (d < D)
            x[d] = (Real)__dadd_rn(a.xmin[d], __dmul_rn((double)x[d], a.xdelta[d]));
        wd_ = __dmul_rn(wd_, xdeltajac);
      }
      w = (Real)wd_;
      if (evaluate) {
        const double f = (double)call_integrand<Real, DMAX, INTEG>(x, D, w, kc, a.params);
        const double tmp = __dmul_rn(wd_, f);  // vflow.py:416
        const double tmp2 = __dmul_rn(tmp, tmp);
        acc1 += tmp;
        acc2 += tmp2;
        if (fill_hist) {
#pragma unroll
          for (int d = 0; d < DMAX; ++d)
            if (d < D) atomicAdd(reinterpret_cast<double*>(my_hist) + d * VF_BINS + ind[d], tmp2);
        }
        if (a.f_out) reinterpret_cast<double*>(a.f_out)[e] = f;
      }
    } else {
      // ---------------- float32 fused form ----------------
      float wf = 1.0f;
      if (a.u_inj != nullptr) {
        // injected float64 uniforms: the index in float64 (bit-exact with the
        // reference), the point and weight in float32.
        const double* up = a.u_inj + e * D;
#pragma unroll
        for (int d = 0; d < DMAX; ++d)
          if (d < D) {
            const double ud = up[d];
            if (vegas) {
              const double xn = __dmul_rn(50.0, __dsub_rn(1.0, ud));
              int i = (int)xn;
              if (i < 0 || i > VF_BINS - 1) {
                bad = 1;
                i = i < 0 ? 0 : VF_BINS - 1;
              }
              const float fr = (float)__dsub_rn(xn, floor(xn));
              const float2 c = cells[d * VF_BINS + i];
              x[d] = (Real)fmaf(c.y, fr, c.x);
              wf = (d == 0) ? c.y : wf * c.y;
              ind[d] = i;
            } else {
              x[d] = (Real)(float)ud;
            }
          }
      } else {
        u32 wd[DMAX];
#pragma unroll
        for (int q = 0; q < (DMAX + 3) / 4; ++q)
          if (4 * q < D) {
            u32 r[4];
            philox_words(ev, a, cw, q, r);
#pragma unroll
            for (int j = 0; j < 4; ++j)
              if (4 * q + j < DMAX) wd[4 * q + j] = r[j];
          }
        if (vegas) {
#pragma unroll
          for (int d = 0; d < DMAX; ++d)
            if (d < D) {
              // t = (~word + 1/2) / 2^32 stands for 1 - u; 50 t = p / 2^32 with
              // p = 50 ~word + 25 exact in 64 bits: bin = p >> 32, fraction = low word.
              const u64 pp = (u64)(~wd[d]) * 50ull + 25ull;
              const int i = (int)(pp >> 32);
              const float fr = frac23((u32)pp);
              const float2 c = cells[d * VF_BINS + i];
              x[d] = (Real)fmaf(c.y, fr, c.x);
              wf = (d == 0) ? c.y : wf * c.y;
              ind[d] = i;
            }
        } else {
#pragma unroll
          for (int d = 0; d < DMAX; ++d)
            if (d < D) x[d] = (Real)(frac23(wd[d]) + 5.9604644775390625e-8f);
        }
      }
      if (limits) {
#pragma unroll
        for (int d = 0; d < DMAX; ++d)
          if (d < D) x[d] = (Real)fmaf((float)x[d], (float)lim[VF_MAX_DIM + d], (float)lim[d]);
      }
      w = (Real)wf;  // the weight without its constant factor (applied in float64 later)
      if (evaluate) {
        const float f = (float)call_integrand<Real, DMAX, INTEG>(x, D, (Real)(wf * wscale_f), kc, a.params);
        const float v = wf * f;
        const float v2 = v * v;
        two_sum_add(s1, v);
        two_sum_add(s2, v2);
        if (fill_hist) {
#pragma unroll
          for (int d = 0; d < DMAX; ++d)
            if (d < D) atomicAdd(reinterpret_cast<float*>(my_hist) + d * VF_BINS + ind[d], v2);
        }
        if (a.f_out) reinterpret_cast<float*>(a.f_out)[e] = f;
      }
    }

    // parity / sample-only taps
    if (a.ind_out && vegas) {
#pragma unroll
      for (int d = 0; d < DMAX; ++d)
        if (d < D) a.ind_out[e * D + d] = ind[d];
    }
    if (a.x_out) {
#pragma unroll
      for (int d = 0; d < DMAX; ++d)
        if (d < D) reinterpret_cast<Real*>(a.x_out)[e * D + d] = x[d];
    }
    if (a.w_out) {
      if constexpr (sizeof(Real) == 8)
        reinterpret_cast<double*>(a.w_out)[e] = (double)w;
      else
        reinterpret_cast<float*>(a.w_out)[e] = (float)((double)w * wscale);
    }
  }

  if (!evaluate) return;  // sample-only launches write no partial rows

  // ---------------- block partials ----------------
  __shared__ double red[2][VF_THREADS / 32];
  double b1, b2;
  if constexpr (sizeof(Real) == 8) {
    acc1 = warp_sum(acc1);
    acc2 = warp_sum(acc2);
    if (lane == 0) {
      red[0][warp] = acc1;
      red[1][warp] = acc2;
    }
  } else {
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if (lane == 0) {
      red[0][warp] = (double)s1.s + (double)s1.c;
      red[1][warp] = (double)s2.s + (double)s2.c;
    }
  }
  if (bad && a.flags) atomicOr(a.flags, VF_FLAG_INDEX_RANGE);
  __syncthreads();

  const int W = 2 + nb;
  double* row = a.partials + (long long)blockIdx.x * W;
  const double scale = wscale;
  if (tid == 0) {
    b1 = 0.0;
    b2 = 0.0;
    for (int i = 0; i < VF_THREADS / 32; ++i) {
      b1 += red[0][i];
      b2 += red[1][i];
    }
    b1 *= scale;
    b2 *= scale * scale;
    if (!isfinite(b1) || !isfinite(b2)) {
      if (a.flags) atomicOr(a.flags, VF_FLAG_NONFINITE);
    }
    if (a.accumulate) {
      row[0] += b1;
      row[1] += b2;
    } else {
      row[0] = b1;
      row[1] = b2;
    }
  }
  if (fill_hist) {
    const double s2c = scale * scale;
    for (int k = tid; k < nb; k += blockDim.x) {
      double h = 0.0;
      for (int c = 0; c < a.hist_copies; ++c) h += (double)hist[c * nb + k];
      h *= s2c;
      if (a.accumulate)
        row[2 + k] += h;
      else
        row[2 + k] = h;
    }
  }
}

}  // namespace vf
