// Device-side building blocks of the VEGAS sampler: the Philox4x32-10 stream,
// uniform conversions, and the built-in integrands.
//
// This header is compiled both ahead of time (nvcc, sm_103a) and at run time
// by NVRTC for user integrands, so it includes no standard headers.
#pragma once

#define VF_BINS 50
#define VF_EDGES 51
#define VF_MAX_DIM 16

// Built-in integrand ids (mirrored in include/vegasflow_gb300.h).
#define VF_INT_NONE 0          // sample only: write x, w, ind; no evaluation
#define VF_INT_SYMGAUSS 1      // prod_d exp(-(x_d-1/2)^2/a^2)/(a sqrt(pi));   params {a, pref}
#define VF_INT_GAUSS 2         // prod_d exp(-(x_d-mu_d)^2/a_d^2);              params {mu[D], a[D]}
#define VF_INT_BREIT_WIGNER 3  // 20000/((s-M^2)^2+M^2 G^2) prod_{d>=1}(1+c_d x_d), s=2500+20000 x_0;
                               //                                              params {M, G, c[D-1]}
#define VF_INT_PROD 4          // prod_d x_d
#define VF_INT_SUM 5           // sum_d x_d
#define VF_INT_USER 99         // NVRTC-compiled user device function

#define VF_FLAG_INDEX_RANGE 1  // an injected uniform mapped outside the grid (clamped)
#define VF_FLAG_REFINE_OVERRUN 2  // the rebinning walk ran past the last bin
#define VF_FLAG_NONFINITE 4    // a partial sum was NaN or Inf
#define VF_FLAG_TIMEOUT 8      // a bounded wait gave up (a copy never completed)
#define VF_FLAG_HISTORY_FULL 16  // an iteration found no history row left (nothing recorded)

namespace vf {

typedef unsigned int u32;
typedef unsigned long long u64;

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Counter layout used by
// every sampler: (ev & 0xffffffff, ev >> 32, (call << 4 | q), call >> 28),
// key = the 64-bit seed.  q selects the 4-word block within one event.
// ---------------------------------------------------------------------------
struct Key {
  u32 k0, k1;
};

__device__ __forceinline__ void philox_round(u32& c0, u32& c1, u32& c2, u32& c3, u32 k0, u32 k1) {
  const u64 p0 = (u64)0xD2511F53u * c0;
  const u64 p1 = (u64)0xCD9E8D57u * c2;
  const u32 hi0 = (u32)(p0 >> 32), lo0 = (u32)p0;
  const u32 hi1 = (u32)(p1 >> 32), lo1 = (u32)p1;
  c0 = hi1 ^ c1 ^ k0;
  c1 = lo1;
  c2 = hi0 ^ c3 ^ k1;
  c3 = lo0;
}

__device__ __forceinline__ void philox4x32_10(u32& c0, u32& c1, u32& c2, u32& c3, Key key) {
  u32 k0 = key.k0, k1 = key.k1;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    philox_round(c0, c1, c2, c3, k0, k1);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// Round keys precomputed on the host (k + r W for r = 0..9): passed in the
// kernel's parameter block, they become constant-bank operands of the xors.
struct RoundKeys {
  u32 k0[10], k1[10];
};

__device__ __forceinline__ void philox4x32_10_rk(u32& c0, u32& c1, u32& c2, u32& c3,
                                                 const RoundKeys& rk) {
#pragma unroll
  for (int r = 0; r < 10; ++r) philox_round(c0, c1, c2, c3, rk.k0[r], rk.k1[r]);
}

// The 4 words of block q of event ev for sampler call `call`.
__device__ __forceinline__ void philox_block(u64 ev, u32 call, u32 q, Key key, u32 w[4]) {
  u32 c0 = (u32)ev, c1 = (u32)(ev >> 32), c2 = (call << 4) | q, c3 = call >> 28;
  philox4x32_10(c0, c1, c2, c3, key);
  w[0] = c0;
  w[1] = c1;
  w[2] = c2;
  w[3] = c3;
}

// 53-bit uniform in [0, 1) from two words.
__device__ __forceinline__ double u53(u32 hi, u32 lo) {
  return __dmul_rn(__dadd_rn(__dmul_rn((double)(hi >> 5), 67108864.0), (double)(lo >> 6)),
                   1.0 / 9007199254740992.0);
}

// The TECH_CUT affine of tf.random.uniform(minval=1e-8, maxval=1-1e-8):
// u * (maxval - minval) + minval, two roundings.
__device__ __forceinline__ double tech_cut(double u) {
  const double range = (1.0 - 1e-8) - 1e-8;
  return __dadd_rn(__dmul_rn(u, range), 1e-8);
}

// float in [0, 1) from the top 23 bits of a word, through the [1, 2) pattern.
__device__ __forceinline__ float frac23(u32 word) {
  return __uint_as_float((word >> 9) | 0x3F800000u) - 1.0f;
}

// ---------------------------------------------------------------------------
// Built-in integrands.  Real = double: the reference's operation order, no FMA
// contraction (parity mode).  Real = float: the fused fp32 form, constants
// prepared once per block (see IntegrandConsts).
// ---------------------------------------------------------------------------
template <typename Real, int DMAX>
struct IntegrandConsts {
  Real c0[DMAX];  // per-dimension constant (mu_d, or c_d)
  Real c1[DMAX];  // per-dimension constant (1/a_d, k_d)
  Real s0, s1, s2;
};

// fp64 parity-mode constants: raw parameters.
template <int DMAX>
__device__ __forceinline__ void load_consts(IntegrandConsts<double, DMAX>& k, int integrand,
                                            const double* __restrict__ p, int D) {
#pragma unroll
  for (int d = 0; d < DMAX; ++d) {
    k.c0[d] = 0.0;
    k.c1[d] = 1.0;
  }
  k.s0 = k.s1 = k.s2 = 0.0;
  if (integrand == VF_INT_SYMGAUSS) {
    k.s0 = p[0];  // a
    k.s1 = p[1];  // pref = (1/a/sqrt(pi))^D
  } else if (integrand == VF_INT_GAUSS) {
#pragma unroll
    for (int d = 0; d < DMAX; ++d)
      if (d < D) {
        k.c0[d] = p[d];
        k.c1[d] = p[D + d];
      }
  } else if (integrand == VF_INT_BREIT_WIGNER) {
    k.s0 = p[0];
    k.s1 = p[1];
#pragma unroll
    for (int d = 1; d < DMAX; ++d)
      if (d < D) k.c0[d] = p[1 + d];
  }
}

// fp32 fused-form constants: folded so the Gaussian is one exp2.
template <int DMAX>
__device__ __forceinline__ void load_consts(IntegrandConsts<float, DMAX>& k, int integrand,
                                            const double* __restrict__ p, int D) {
  const double LOG2E = 1.4426950408889634;
#pragma unroll
  for (int d = 0; d < DMAX; ++d) {
    k.c0[d] = 0.0f;
    k.c1[d] = 1.0f;
  }
  k.s0 = k.s1 = k.s2 = 0.0f;
  if (integrand == VF_INT_SYMGAUSS) {
    // exp(-sum((x-1/2)/a)^2) = exp2(-sum(((x-1/2) k)^2)), k = sqrt(log2 e)/a
    const float kk = (float)(sqrt(LOG2E) / p[0]);
#pragma unroll
    for (int d = 0; d < DMAX; ++d) {
      k.c0[d] = (float)(-0.5 * (sqrt(LOG2E) / p[0]));  // -mu k
      k.c1[d] = kk;
    }
    k.s1 = (float)p[1];
  } else if (integrand == VF_INT_GAUSS) {
#pragma unroll
    for (int d = 0; d < DMAX; ++d)
      if (d < D) {
        const double kd = sqrt(LOG2E) / p[D + d];
        k.c0[d] = (float)(-p[d] * kd);
        k.c1[d] = (float)kd;
      }
    k.s1 = 1.0f;
  } else if (integrand == VF_INT_BREIT_WIGNER) {
    const double m2 = p[0] * p[0];
    k.s0 = (float)(2500.0 - m2);        // s - M^2 = 20000 x_0 + (2500 - M^2)
    k.s2 = (float)(m2 * p[1] * p[1]);   // M^2 G^2
#pragma unroll
    for (int d = 1; d < DMAX; ++d)
      if (d < D) k.c0[d] = (float)p[1 + d];
  }
}

template <int DMAX>
__device__ __forceinline__ double eval_builtin(int integrand, const double* x, int D,
                                               const IntegrandConsts<double, DMAX>& k) {
  double f = 0.0;
  if (integrand == VF_INT_SYMGAUSS) {
    double coef = 0.0;
#pragma unroll
    for (int d = 0; d < DMAX; ++d)
      if (d < D) {
        const double t = __dsub_rn(x[d], 0.5) / k.s0;
        coef = __dadd_rn(coef, __dmul_rn(t, t));
      }
    f = __dmul_rn(k.s1, exp(-coef));
  } else if (integrand == VF_INT_GAUSS) {
    double coef = 0.0;
#pragma unroll
    for (int d = 0; d < DMAX; ++d)
      if (d < D) {
        const double t = __dsub_rn(x[d], k.c0[d]) / k.c1[d];
        coef = __dadd_rn(coef, __dmul_rn(t, t));
      }
    f = exp(-coef);
  } else if (integrand == VF_INT_BREIT_WIGNER) {
    const double s = __dadd_rn(2500.0, __dmul_rn(20000.0, x[0]));
    const double m2 = __dmul_rn(k.s0, k.s0);
    const double ds = __dsub_rn(s, m2);
    f = 20000.0 / __dadd_rn(__dmul_rn(ds, ds), __dmul_rn(__dmul_rn(m2, k.s1), k.s1));
#pragma unroll
    for (int d = 1; d < DMAX; ++d)
      if (d < D) f = __dmul_rn(f, __dadd_rn(1.0, __dmul_rn(k.c0[d], x[d])));
  } else if (integrand == VF_INT_PROD) {
    f = x[0];
#pragma unroll
    for (int d = 1; d < DMAX; ++d)
      if (d < D) f = __dmul_rn(f, x[d]);
  } else if (integrand == VF_INT_SUM) {
    f = x[0];
#pragma unroll
    for (int d = 1; d < DMAX; ++d)
      if (d < D) f = __dadd_rn(f, x[d]);
  }
  return f;
}

template <int DMAX>
__device__ __forceinline__ float eval_builtin(int integrand, const float* x, int D,
                                              const IntegrandConsts<float, DMAX>& k) {
  float f = 0.0f;
  if (integrand == VF_INT_SYMGAUSS || integrand == VF_INT_GAUSS) {
    float coef = 0.0f;
#pragma unroll
    for (int d = 0; d < DMAX; ++d)
      if (d < D) {
        const float t = fmaf(x[d], k.c1[d], k.c0[d]);
        coef = fmaf(t, t, coef);
      }
    f = k.s1 * exp2f(-coef);
  } else if (integrand == VF_INT_BREIT_WIGNER) {
    const float ds = fmaf(20000.0f, x[0], k.s0);
    f = 20000.0f / fmaf(ds, ds, k.s2);
#pragma unroll
    for (int d = 1; d < DMAX; ++d)
      if (d < D) f *= fmaf(k.c0[d], x[d], 1.0f);
  } else if (integrand == VF_INT_PROD) {
    f = x[0];
#pragma unroll
    for (int d = 1; d < DMAX; ++d)
      if (d < D) f *= x[d];
  } else if (integrand == VF_INT_SUM) {
    f = x[0];
#pragma unroll
    for (int d = 1; d < DMAX; ++d)
      if (d < D) f += x[d];
  }
  return f;
}

// ---------------------------------------------------------------------------
// Compensated fp32 accumulation (Knuth's TwoSum): s + c carries the exact sum
// of everything added, to within one rounding of c.
// ---------------------------------------------------------------------------
struct F2 {
  float s, c;
};

__device__ __forceinline__ void two_sum_add(F2& a, float v) {
  const float s = a.s + v;
  const float bb = s - a.s;
  const float err = (a.s - (s - bb)) + (v - bb);
  a.s = s;
  a.c += err;
}

__device__ __forceinline__ F2 two_sum_merge(F2 a, F2 b) {
  F2 r;
  r.s = a.s + b.s;
  const float bb = r.s - a.s;
  const float err = (a.s - (r.s - bb)) + (b.s - bb);
  r.c = a.c + b.c + err;
  return r;
}

}  // namespace vf
