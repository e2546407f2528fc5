// The fused fp32 VEGAS samplers: the performance path of the float32 form.
//
// Two kernels, both specialised at compile time on the exact dimension count
// and the integrand, reading nothing per event from HBM but their inputs:
//
//   vf_vegas_f32_kernel      in-kernel Philox4x32-10 uniforms (the benchmarked
//                            path, C2's fp32 form)
//   vf_vegas_f32_inj_kernel  injected float64 uniforms streamed from HBM by TMA
//                            tiles (C2's injected mode)
//
// Per event and dimension one fused multiply-add through a per-bin table
// {C0, C1} staged in shared memory, which folds the importance map, the
// integration limits and -- for the Gaussian family -- the integrand's affine
// argument:
//
//   generic integrand:  x = c0 + c1 (1 + frac),  c0 = xmin + (lo - delta) xdelta,
//                       c1 = delta xdelta  (frac: the reference's fractional bin
//                       coordinate, vflow.py:75-76)
//   Gaussian family:    t = (x - mu) sqrt(log2 e) / a as the same affine map,
//                       f = 2^(-sum t^2)  (the normalisation goes to the float64
//                       scale)
//   weight w = 2^kw prod_d c1 (float32, kw a per-block power-of-two prescale
//   that keeps a typical event's weight near 1 at any dimension count); the
//   constant 50^D xjac 2^-kw (* pref / prod k) is applied in float64 to the
//   block partials.
//
// Philox kernel.  A word w stands for the uniform u = (w + 1/2) / 2^32, whose
// reference bin is trunc(50 (1 - u)) (vflow.py:117, :67).  p = 50 w + 25 is
// 50 u 2^32 exactly (64-bit), so j = p >> 32 = floor(50 u) and the reference bin
// is 49 - j (50 u is never an integer); its fraction 1 - frac(50 u) comes from
// p's low word.  The table is therefore stored in reversed bin order, cell j
// holding bin 49 - j as C0 = c0 + 3 c1, C1 = -c1 (computed in float64, rounded
// once), so that with m = 1 + (the top 23 bits of p mod 2^32) / 2^23 in [1, 2):
//       C0 + C1 m = c0 + c1 (2 - frac(50 u)) = c0 + c1 (1 + frac(50 (1 - u)))
// -- one 64-bit multiply-add, two bit operations and one table lookup per
// dimension, no complement.  The weight's sign (-1)^D goes to the float64 scale.
//
// The table is replicated VF_F32_TC = 16 times, copy c in bank pair c: lane l
// reads copy l % 16, so the 64-bit lookups of a half-warp never share a bank
// (2 shared-memory wavefronts per warp lookup instead of ~7 with one copy; the
// shared-memory pipe is what the histogram atomics compete for).
//
// Per event: TwoSum-compensated fp32 sums of w f and (w f)^2, and (when
// training) the (w f)^2 histogram in joint tables of dimension pairs: dims
// (0,1), (2,3), ... share one table of 50 rows per block, so an event makes
// ceil(D/2) float atomic additions (compare-and-swap loops on this part)
// instead of D.  Rows are VF_F32_JOINT_ROW floats: 64 with the column index
// XOR-swizzled by the row's low bits (the cell address is shifts and a logical
// operation, and a warp's random cells spread evenly over the banks), or 50.
// At the end each dimension's 50 bins are its pair table's row or column sums
// (an odd last dimension has a plain 50-bin table).
#pragma once
#include "vf_sample.cuh"

// lane-replicated copies of the per-bin table (Philox kernel)
#define VF_F32_TC 16

// floats per row of a joint pair table (64: XOR-swizzled columns; 50: plain)
#ifndef VF_F32_JOINT_ROW
#define VF_F32_JOINT_ROW 64
#endif

namespace vf {

__device__ __forceinline__ float ex2_approx_ftz(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// floats of the 50 x 50 joint tables (plus a plain table for an odd last
// dimension) with 50-float rows: the batched sampler and the injected kernel
__host__ __device__ inline int vegas_f32_joint_floats(int D) { return (D / 2) * 2500 + (D & 1) * 50; }

// The Philox kernel's joint tables: rows of VF_F32_JOINT_ROW floats.
__host__ __device__ constexpr int vegas_f32_pair_floats() { return VF_BINS * VF_F32_JOINT_ROW; }
__host__ __device__ inline int vegas_f32_hist_floats(int D) {
  return (D / 2) * vegas_f32_pair_floats() + (D & 1) * VF_BINS;
}
__host__ __device__ inline int vegas_f32_table_bytes(int D) { return D * VF_BINS * VF_F32_TC * 8; }

// Dynamic shared memory of the Philox kernel.
__host__ __device__ inline int vegas_f32_smem_bytes(int D, int train) {
  return vegas_f32_table_bytes(D) + (train ? vegas_f32_hist_floats(D) * 4 : 0);
}

// Offset of cell (row r, column c) of a joint pair table.
__device__ __forceinline__ int joint_cell(int r, int c) {
  if (VF_F32_JOINT_ROW == 64)
    return (r << 6) + (c ^ (r & 31));
  else
    return r * VF_F32_JOINT_ROW + c;
}

// The reference's bin of an injected float64 uniform u, ind = trunc(fl(50 *
// fl(1 - u))) (vflow.py:117, :67), without float64 arithmetic: for u in
// [2^-12, 1), U = u 2^64 is an exact 64-bit integer and y = 50 (1 - u) is
// exactly 50 (2^64 - U) / 2^64.  With h = the high word of U, P = 50 (2^32 - 1 - h)
// is a 38-bit integer and y 2^32 = P + c, c in [0, 50] (c holds the low word's
// share).  So when the low 32 bits f of P lie in [1, 2^32 - 52], adding c neither
// carries into the integer part nor lands within 2^-32 of an integer: ind = P >> 32
// is trunc(y), and the reference's two roundings (which move y by less than
// 100 2^-53 < 2^-46) cannot change it.  Otherwise (f within 52 of an integer
// boundary, about 1 uniform in 8e7) -- and for every u outside [2^-12, 1), NaN,
// negative, >= 1 -- the caller repeats the float64 operations.  m = 1 + f's top
// 23 bits (below 1 + the true fraction by less than 2^-23 + 51 2^-32).  About 10
// 32-bit operations per uniform.  Returns false for the float64 cases.
// Branch-free form of inj_bin_exact for the fast path of a whole event: ind
// and m are computed whatever the input (ind stays in 0..49: P < 50 2^32) and
// the return value says whether they are the reference's; the caller redoes
// the event's failing uniforms (rare) with the exact operations.
__device__ __forceinline__ bool inj_bin_fast(u64 bits, int& ind, float& m) {
  const u32 bh = (u32)(bits >> 32), bl = (u32)bits;
  const u32 sh = (bh >> 20) - 1011u;
  const u32 mh = (bh & 0xFFFFFu) | 0x100000u;
  const u32 h = __funnelshift_l(bl, mh, sh);
  const u64 P = (u64)(~h) * 50ull;
  const u32 f = (u32)P;
  ind = (int)(P >> 32);
  m = __uint_as_float(__funnelshift_r(f, 0x7Fu, 9));
  return (sh <= 11u) & (f - 1u < 0xFFFFFFCCu);
}

__device__ __forceinline__ bool inj_bin_exact(u64 bits, int& ind, float& m) {
  const u32 bh = (u32)(bits >> 32), bl = (u32)bits;
  const u32 sh = (bh >> 20) - 1011u;  // biased exponent - 1011: u in [2^-12, 1) <=> sh in [0, 11]
  if (sh > 11u) return false;
  const u32 mh = (bh & 0xFFFFFu) | 0x100000u;  // the mantissa's high word, implicit bit set
  const u32 h = __funnelshift_l(bl, mh, sh);   // high word of U = mantissa << sh
  const u64 P = (u64)(~h) * 50ull;
  const u32 f = (u32)P;
  if (f - 1u >= 0xFFFFFFCCu) return false;  // f outside [1, 2^32 - 52]
  ind = (int)(P >> 32);
  m = __uint_as_float(__funnelshift_r(f, 0x7Fu, 9));  // 0x3F800000 | (f >> 9)
  return true;
}

// ---- TMA staging of injected uniforms
__device__ __forceinline__ u32 smem_u32(const void* p) { return (u32)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(u32 bar, u32 count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// One tile: the barrier expects `bytes`, the tensor copy completes them.
__device__ __forceinline__ void tma_load_tile(u32 dst, const void* tmap, int x, int y, u32 bar, u32 bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<unsigned long long>(tmap)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Wait for phase `parity` of the barrier, giving up after `polls` polls (the
// default is about a tenth of a second); returns whether the phase completed.
__device__ __forceinline__ bool mbar_wait_bounded(u32 bar, u32 parity, int polls = 1 << 20) {
  for (int i = 0; i < polls; ++i) {
    u32 ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (i >= 16) __nanosleep(64);
  }
  return false;
}

// ---- per-block constants and the per-bin table, shared by both kernels

// The float64 weight constant 50^D xjac (* pref / prod k for the Gaussian
// family), times `sign`; thread 0 writes it, the caller syncs before reading it.
template <int D, bool GAUSS, int INTEG>
__device__ __forceinline__ void f32_block_constants(const SampleArgs& a, double* g_mu, double* g_k, double* g_wscale,
                                                    double sign) {
  constexpr double SQRT_LOG2E = 1.2011224087864498;  // sqrt(log2(e))
  const int tid = threadIdx.x;
  if (GAUSS && tid < D) {
    g_mu[tid] = (INTEG == VF_INT_SYMGAUSS) ? 0.5 : a.params[tid];
    g_k[tid] = SQRT_LOG2E / ((INTEG == VF_INT_SYMGAUSS) ? a.params[0] : a.params[D + tid]);
  }
  __syncthreads();
  if (tid == 0) {
    double ws = a.xjac * sign;
    for (int d = 0; d < D; ++d) ws *= 50.0;
    if (GAUSS) {
      double prodk = 1.0;
      for (int d = 0; d < D; ++d) prodk *= g_k[d];
      ws *= ((INTEG == VF_INT_SYMGAUSS) ? a.params[1] : 1.0) / prodk;
    }
    *g_wscale = ws;
  }
}

// The affine coefficients (c0, c1) of bin b of dimension d, in float64.
template <bool GAUSS>
__device__ __forceinline__ void f32_bin_affine(const SampleArgs& a, const double* g_mu, const double* g_k, int d,
                                               int b, double& c0, double& c1) {
  const double lo = a.grid[d * VF_EDGES + b];
  const double dl = a.grid[d * VF_EDGES + b + 1] - lo;
  c0 = lo - dl;
  c1 = dl;
  if (a.xmin != nullptr) {
    c0 = __fma_rn(c0, a.xdelta[d], a.xmin[d]);
    c1 = c1 * a.xdelta[d];
  }
  if (GAUSS) {
    c0 = (c0 - g_mu[d]) * g_k[d];
    c1 = c1 * g_k[d];
  }
}

// Binary exponent of |c1| (bounded to float32's normal range; a zero-width bin
// counts as the smallest), for the weight prescale below.
__device__ __forceinline__ int f32_cell_exponent(double c1) {
  const int e = (int)((__double_as_longlong(c1) >> 52) & 0x7FF) - 1023;
  return e < -126 ? -126 : (e > 127 ? 127 : e);
}

// The power-of-two prescale of the fp32 weight.  An event's weight prod_d c1
// can leave float32's range at large dimension counts (prod_d delta ~ 50^-D on
// a uniform grid: 6.6e-28 at D = 16, whose square underflows), so the kernels
// accumulate (S w f) and (S w f)^2 with S = 2^k, k = -round(sum_d mean_b
// log2 |c1_db|) from the cells' binary exponents (`expsum`: their sum over
// all D x 50 cells): the weight of a typical event -- the bins are equally
// likely -- is then about 1.  Returns k; the float64 scale takes 2^-k back,
// so the scaling is exact.
__device__ __forceinline__ int f32_prescale_exponent(int expsum) {
  int k = -__float2int_rn((float)expsum / (float)VF_BINS);
  return k < -100 ? -100 : (k > 100 ? 100 : k);
}

// Block-wide sum of the per-thread exponent sums into *acc (zeroed before the
// block's first barrier): a warp reduction, then one shared atomic per warp.
__device__ __forceinline__ void f32_add_exponents(int* acc, int mine) {
  mine = __reduce_add_sync(0xffffffffu, mine);
  if ((threadIdx.x & 31) == 0) atomicAdd(acc, mine);
}

// ---- the Philox kernel -------------------------------------------------------

// THREADS: the block size (1024 or 512; the launch-shape autotuner chooses),
// with registers capped at 64 per thread (one 1024-thread or two 512-thread
// blocks per SM).  TAP: the parity instantiation, which also writes every
// event's D bin indices to a.ind_out ([n_events][D] int32); the kernels of the
// hot path are TAP = false, where the writes do not exist.
template <int D, int INTEG, int THREADS, bool TAP = false>
__global__ void __launch_bounds__(THREADS, (THREADS >= 1024 ? 1 : 2048 / THREADS))
vf_vegas_f32_kernel(const __grid_constant__ SampleArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NB = D * VF_BINS;
  constexpr int NP = D / 2;
  constexpr int PAIR = vegas_f32_pair_floats();
  constexpr int DSTRIDE = VF_BINS * VF_F32_TC * 8;  // bytes per dimension of the table
  constexpr bool GAUSS = (INTEG == VF_INT_SYMGAUSS || INTEG == VF_INT_GAUSS);
  float2* cells = reinterpret_cast<float2*>(smem);
  float* hist = reinterpret_cast<float*>(smem + vegas_f32_table_bytes(D));
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const bool train = a.train != 0;
  const CallWords cw = call_words(a);

  // ---- per-block float64 constants; the reversed, replicated table; histograms
  __shared__ double g_mu[D], g_k[D], g_wscale;
  __shared__ int g_expsum;
  if (tid == 0) g_expsum = 0;
  f32_block_constants<D, GAUSS, INTEG>(a, g_mu, g_k, &g_wscale, (D & 1) ? -1.0 : 1.0);
  int expsum = 0;
  for (int k = tid; k < NB; k += THREADS) {
    const int d = k / VF_BINS, b = k - d * VF_BINS;
    double c0, c1;
    f32_bin_affine<GAUSS>(a, g_mu, g_k, d, b, c0, c1);
    expsum += f32_cell_exponent(c1);
    const float2 cell = make_float2((float)__fma_rn(3.0, c1, c0), (float)(-c1));
    float2* dst = cells + (d * VF_BINS + (VF_BINS - 1 - b)) * VF_F32_TC;
#pragma unroll
    for (int c = 0; c < VF_F32_TC; ++c) dst[c] = cell;
  }
  f32_add_exponents(&g_expsum, expsum);
  if (train)
    for (int k = tid; k < vegas_f32_hist_floats(D); k += THREADS) hist[k] = 0.0f;
  __syncthreads();

  // the weight prescale 2^kw (exact), taken back by the float64 scale, which
  // also holds the weight's sign (-1)^D
  const int kw = f32_prescale_exponent(g_expsum);
  const float wpre = __int_as_float((127 + kw) << 23);
  const double wscale = g_wscale * ldexp(1.0, -kw);
  [[maybe_unused]] const float wscale_f = (float)wscale;
  IntegrandConsts<float, D> kc;
  if (!GAUSS) load_consts<D>(kc, INTEG == VF_INT_USER ? VF_INT_NONE : INTEG, a.params, D);
  // this lane's copy of the table
  const char* mytab = reinterpret_cast<const char*>(cells + (lane & (VF_F32_TC - 1)));
  F2 s1 = {0.0f, 0.0f}, s2 = {0.0f, 0.0f};

  // one event's Philox words -> table cells j (reference bin 49 - j), weight,
  // and the Gaussian exponent (or x)
  auto draw = [&](u64 ev, int (&bins)[D], float& wf, float& s, float (&x)[D]) {
#pragma unroll
    for (int q = 0; q < (D + 3) / 4; ++q) {
      u32 c0 = (u32)ev, c1 = (u32)(ev >> 32), c2 = cw.c2base | (u32)q, c3 = cw.c3;
      philox4x32_10_rk(c0, c1, c2, c3, a.rk);
      const u32 wq[4] = {c0, c1, c2, c3};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int d = 4 * q + j;
        if (d < D) {
          const u64 pp = (u64)wq[j] * 50ull + 25ull;
          const u32 jj = (u32)(pp >> 32);
          const float m = __uint_as_float(((u32)pp >> 9) | 0x3F800000u);
          const float2 c = *reinterpret_cast<const float2*>(mytab + (jj << 7) + d * DSTRIDE);
          const float t = fmaf(c.y, m, c.x);
          wf = (d == 0) ? wpre * c.y : wf * c.y;
          if (GAUSS)
            s = fmaf(t, t, s);
          else
            x[d] = t;
          bins[d] = (int)jj;
        }
      }
    }
  };

  // one event from its cells: the integrand, the sums and the histogram
  auto finish = [&](const int (&bins)[D], float wf, float s, const float (&x)[D]) {
    float f;
    if constexpr (GAUSS) {
      f = ex2_approx_ftz(-s);
    } else {
#ifdef VF_JIT_USER
      if constexpr (INTEG == VF_INT_USER)
        f = (float)VF_USER_FN(x, D, wf * wscale_f, a.params);
      else
#endif
        f = eval_builtin<D>(INTEG, x, D, kc);
    }
    const float v = wf * f;
    const float v2 = v * v;
    two_sum_add(s1, v);
    two_sum_add(s2, v2);
    if (train) {
#pragma unroll
      for (int p = 0; p < NP; ++p) atomicAdd(hist + p * PAIR + joint_cell(bins[2 * p], bins[2 * p + 1]), v2);
      if (D & 1) atomicAdd(hist + NP * PAIR + bins[D - 1], v2);
    }
  };

  // parity tap: the reference's bin indices of the event
  auto tap = [&](long long e, const int (&bins)[D]) {
    if constexpr (TAP) {
#pragma unroll
      for (int d = 0; d < D; ++d) a.ind_out[e * D + d] = VF_BINS - 1 - bins[d];
    }
  };

  const long long n = a.n_events;
  const long long stride = (long long)gridDim.x * THREADS;
  long long e = (long long)blockIdx.x * THREADS + tid;
  // Two events per pass give the scheduler two independent draws to overlap
  // (shared-memory latency of one with the Philox rounds of the other); the
  // registers it needs pay for themselves only at small D.
  if constexpr (D <= 4) {
    for (; e + stride < n; e += 2 * stride) {
      const u64 ev0 = (u64)(a.ev_offset + e), ev1 = ev0 + (u64)stride;
      int b0[D], b1[D];
      float x0[D], x1[D];
      float wf0 = 1.0f, s0 = 0.0f, wf1 = 1.0f, s1_ = 0.0f;
      draw(ev0, b0, wf0, s0, x0);
      draw(ev1, b1, wf1, s1_, x1);
      finish(b0, wf0, s0, x0);
      finish(b1, wf1, s1_, x1);
      tap(e, b0);
      tap(e + stride, b1);
    }
  }
  for (; e < n; e += stride) {
    int bins[D];
    float x[D];
    float wf = 1.0f, s = 0.0f;
    draw((u64)(a.ev_offset + e), bins, wf, s, x);
    finish(bins, wf, s, x);
    tap(e, bins);
  }

  // ---- block partials: TwoSum merges across the warp and the block, float64 row
  __shared__ double red[2][THREADS / 32];
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  if (lane == 0) {
    red[0][warp] = (double)s1.s + (double)s1.c;
    red[1][warp] = (double)s2.s + (double)s2.c;
  }
  __syncthreads();
  const int W = 2 + NB;
  double* row = a.partials + (long long)blockIdx.x * W;
  if (tid == 0) {
    double b1 = 0.0, b2 = 0.0;
    for (int i = 0; i < THREADS / 32; ++i) {
      b1 += red[0][i];
      b2 += red[1][i];
    }
    b1 *= wscale;
    b2 *= wscale * wscale;
    if ((!isfinite(b1) || !isfinite(b2)) && a.flags) atomicOr(a.flags, VF_FLAG_NONFINITE);
    if (a.accumulate) {
      row[0] += b1;
      row[1] += b2;
    } else {
      row[0] = b1;
      row[1] = b2;
    }
  }
  if (train) {
    // marginals in fp32 (the tables are fp32), one float64 scaling per bin;
    // bin b of a dimension is its table's cell 49 - b
    const double s2c = wscale * wscale;
    for (int k = tid; k < NB; k += THREADS) {
      const int d = k / VF_BINS, b = k - d * VF_BINS;
      const int jb = VF_BINS - 1 - b;
      float hf = 0.0f;
      if (d < 2 * NP) {
        const float* tab = hist + (d >> 1) * PAIR;
        if ((d & 1) == 0)
          for (int c = 0; c < VF_F32_JOINT_ROW; ++c) hf += tab[jb * VF_F32_JOINT_ROW + c];  // row sum
        else
          for (int r = 0; r < VF_BINS; ++r) hf += tab[joint_cell(r, jb)];  // column sum
      } else {
        hf = hist[NP * PAIR + jb];
      }
      const double h = (double)hf * s2c;
      if (a.accumulate)
        row[2 + k] += h;
      else
        row[2 + k] = h;
    }
  }
  // rows beyond the grid (a launch with fewer blocks than the caller's rows)
  if (!a.accumulate)
    for (long long r = blockIdx.x + (long long)gridDim.x; r < a.rows_total; r += gridDim.x)
      for (int k = tid; k < W; k += THREADS) a.partials[r * W + k] = 0.0;
}

// ---- the injected-uniform kernel ----------------------------------------------
//
// Injected float64 uniforms ([n][D] row-major, streamed once) with the
// reference's float64 bin of every uniform (inj_bin_exact, or the float64
// operations in its rare cases).  1024 threads per block (one block per SM).
// With a.tma_swizzle set (D = 4, 8, 16 and a 16-byte aligned array) every warp
// streams its own tiles of VF_INJ_ROWS = 32 events (lane r takes row r)
// through a ring of `stages` shared-memory stages filled by TMA tensor copies
// (the tensor map's 32/64/128-byte swizzle makes every quarter-warp read of a
// row conflict-free): the lanes copy their rows to registers, meet at a warp
// barrier that also votes on the wait, lane 0 issues the copy of the tile
// `stages` ahead into the freed stage, and the events are evaluated while the
// copies land -- 32 warps keep up to 32 `stages` tiles (64-128 KB) in flight
// per SM, and no warp waits for another.  Otherwise plain loads (16-byte,
// evict-first when D is even and the array is aligned).
// The bin table is lane-replicated as in the Philox kernel but in bin order,
// the histogram joint pair tables have 50-float rows.

#define VF_INJ_THREADS 1024
#define VF_INJ_ROWS 32
#define VF_INJ_GROUPS (VF_INJ_THREADS / VF_INJ_ROWS)
#define VF_SMEM_LIMIT 232448  // dynamic shared memory a block may use (227 KB)

// Table copies and stages per group of the injected kernel for dimension D
// (the largest that fit in shared memory; stages = 0: no TMA path for this D).
// With the TMA ring, 1024 bytes of slack in front of it let the ring start on
// a 1024-byte boundary wherever the dynamic shared memory begins.
__host__ __device__ constexpr int inj_tma_dim(int D) { return D == 4 || D == 8 || D == 16; }
__host__ __device__ constexpr int inj_table_bytes(int D, int tc) { return D * VF_BINS * tc * 8; }
__host__ __device__ constexpr int inj_hist_bytes(int D) { return ((D / 2) * 2500 + (D & 1) * VF_BINS) * 4; }
__host__ __device__ constexpr int inj_tile_bytes(int D) { return VF_INJ_ROWS * 8 * D; }
__host__ __device__ constexpr int inj_fit(int D, int tc, int st) {
  return inj_table_bytes(D, tc) + inj_hist_bytes(D) + (st ? 1024 : 0) + VF_INJ_GROUPS * st * inj_tile_bytes(D) <=
         VF_SMEM_LIMIT;
}
__host__ __device__ constexpr int inj_tc(int D) {
  return !inj_tma_dim(D) ? (inj_fit(D, 16, 0) ? 16 : 1)
                         : (inj_fit(D, 16, 2) ? 16 : (inj_fit(D, 1, 2) ? 1 : (inj_fit(D, 16, 1) ? 16 : 1)));
}
__host__ __device__ constexpr int inj_stages(int D) {
  return !inj_tma_dim(D) ? 0 : (inj_fit(D, inj_tc(D), 2) ? 2 : 1);
}
// Dynamic shared memory of the injected kernel: table and histogram, and with
// `tma` the stage ring (with its 1024 bytes of slack).
__host__ __device__ inline int vegas_f32_inj_smem_bytes(int D, int train, bool tma = false) {
  const int base = inj_table_bytes(D, inj_tc(D)) + (train ? inj_hist_bytes(D) : 0);
  if (!tma || !inj_tma_dim(D)) return base;
  return base + 1024 + VF_INJ_GROUPS * inj_stages(D) * inj_tile_bytes(D);
}

template <int D, int INTEG, bool TAP = false>
__global__ void __launch_bounds__(VF_INJ_THREADS, 1) vf_vegas_f32_inj_kernel(const __grid_constant__ SampleArgs a) {
  constexpr int THREADS = VF_INJ_THREADS;
  constexpr int TC = inj_tc(D);
  constexpr int STAGES = inj_stages(D);
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NB = D * VF_BINS;
  constexpr int NP = D / 2;
  constexpr int DSTRIDE = VF_BINS * TC * 8;
  constexpr bool GAUSS = (INTEG == VF_INT_SYMGAUSS || INTEG == VF_INT_GAUSS);
  float2* cells = reinterpret_cast<float2*>(smem);
  float* hist = reinterpret_cast<float*>(smem + inj_table_bytes(D, TC));
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const bool train = a.train != 0;

  // the TMA path's barriers: one per stage of every warp, initialised before
  // the block-wide sync below
  __shared__ alignas(8) u64 tma_bar[VF_INJ_GROUPS][STAGES > 0 ? STAGES : 1];
  const bool tma = STAGES > 0 && a.tma_swizzle != 0;
  if (tma && tid == 0) {
    for (int gg = 0; gg < VF_INJ_GROUPS; ++gg)
      for (int st = 0; st < STAGES; ++st) mbar_init(smem_u32(&tma_bar[gg][st]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __shared__ double g_mu[D], g_k[D], g_wscale;
  __shared__ int g_expsum;
  if (tid == 0) g_expsum = 0;
  f32_block_constants<D, GAUSS, INTEG>(a, g_mu, g_k, &g_wscale, 1.0);
  int expsum = 0;
  for (int k = tid; k < NB; k += THREADS) {
    const int d = k / VF_BINS, b = k - d * VF_BINS;
    double c0, c1;
    f32_bin_affine<GAUSS>(a, g_mu, g_k, d, b, c0, c1);
    expsum += f32_cell_exponent(c1);
    const float2 cell = make_float2((float)c0, (float)c1);
#pragma unroll
    for (int c = 0; c < TC; ++c) cells[k * TC + c] = cell;
  }
  f32_add_exponents(&g_expsum, expsum);
  if (train)
    for (int k = tid; k < inj_hist_bytes(D) / 4; k += THREADS) hist[k] = 0.0f;
  __syncthreads();  // constants, table, histogram and barriers ready

  const int kw = f32_prescale_exponent(g_expsum);  // the weight prescale, as in the Philox kernel
  const float wpre = __int_as_float((127 + kw) << 23);
  const double wscale = g_wscale * ldexp(1.0, -kw);
  [[maybe_unused]] const float wscale_f = (float)wscale;
  IntegrandConsts<float, D> kc;
  if (!GAUSS) load_consts<D>(kc, INTEG == VF_INT_USER ? VF_INT_NONE : INTEG, a.params, D);
  const char* mytab = reinterpret_cast<const char*>(cells + (lane & (TC - 1)));
  F2 s1 = {0.0f, 0.0f}, s2 = {0.0f, 0.0f};
  int bad = 0;

  // the bin and fraction of one uniform exactly (the rare cases of the integer
  // map: the reference's float64 operations, vflow.py:117, :67)
  auto exact_bin = [&](u64 ub, int& i, float& m) {
    if (!inj_bin_exact(ub, i, m)) {
      const double xn = __dmul_rn(50.0, __dsub_rn(1.0, __longlong_as_double((long long)ub)));
      i = (int)xn;
      if (i < 0 || i > VF_BINS - 1) {
        bad = 1;
        i = i < 0 ? 0 : VF_BINS - 1;
      }
      m = (float)(1.0 + (xn - floor(xn)));
    }
  };
  // the event's dimensions through the table, the bins by the fast integer map
  // or (`exact`) the exact one; returns whether every bin came out exact
  auto map_dims = [&](const u64 (&ub)[D], int (&bins)[D], float& wf, float& s, float (&x)[D], bool exact) {
    bool ok = true;
    wf = 1.0f;
    s = 0.0f;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      int i;
      float m;
      if (exact)
        exact_bin(ub[d], i, m);
      else
        ok &= inj_bin_fast(ub[d], i, m);
      const float2 c = *reinterpret_cast<const float2*>(mytab + i * (TC * 8) + d * DSTRIDE);
      const float t = fmaf(c.y, m, c.x);
      wf = (d == 0) ? wpre * c.y : wf * c.y;
      if (GAUSS)
        s = fmaf(t, t, s);
      else
        x[d] = t;
      bins[d] = i;
    }
    return ok;
  };

  auto event = [&](const u64 (&ub)[D], long long e) {
    int bins[D];
    float x[D];
    float wf, s;
    // every uniform by the integer map, one check for the event; an event with
    // a uniform the map cannot decide (about one in 1e7 at D = 8 on U[0, 1)
    // uniforms) is mapped again with the exact operations
    if (!map_dims(ub, bins, wf, s, x, false)) map_dims(ub, bins, wf, s, x, true);
    float f;
    if constexpr (GAUSS) {
      f = ex2_approx_ftz(-s);
    } else {
#ifdef VF_JIT_USER
      if constexpr (INTEG == VF_INT_USER)
        f = (float)VF_USER_FN(x, D, wf * wscale_f, a.params);
      else
#endif
        f = eval_builtin<D>(INTEG, x, D, kc);
    }
    const float v = wf * f;
    const float v2 = v * v;
    two_sum_add(s1, v);
    two_sum_add(s2, v2);
    if (train) {
#pragma unroll
      for (int p = 0; p < NP; ++p) atomicAdd(hist + p * 2500 + bins[2 * p] * VF_BINS + bins[2 * p + 1], v2);
      if (D & 1) atomicAdd(hist + NP * 2500 + bins[D - 1], v2);
    }
    if constexpr (TAP) {
#pragma unroll
      for (int d = 0; d < D; ++d) a.ind_out[e * D + d] = bins[d];
    }
  };

  const long long n = a.n_events;
  if constexpr (STAGES > 0) {
    if (tma) {
      constexpr int ROWB = 8 * D;
      constexpr u32 TILEB = inj_tile_bytes(D);  // 1, 2 or 4 KB: every stage on a 1 KB boundary
      const u32 ring = (smem_u32(smem) + (u32)vegas_f32_inj_smem_bytes(D, a.train) + 1023u) & ~1023u;
      const int g = warp, r = lane;
      const u32 stage0 = ring + (u32)(g * STAGES) * TILEB;
      const long long n_tiles = (n + VF_INJ_ROWS - 1) / VF_INJ_ROWS;
      // the warp's tiles: first, first + step, ...
      const long long step = (long long)gridDim.x * VF_INJ_GROUPS;
      const long long first = (long long)blockIdx.x * VF_INJ_GROUPS + g;
      if (r == 0)
        for (int st = 0; st < STAGES; ++st) {
          const long long t = first + st * step;
          if (t < n_tiles)
            tma_load_tile(stage0 + (u32)st * TILEB, a.tmap, 0, (int)(t * VF_INJ_ROWS), smem_u32(&tma_bar[g][st]),
                          TILEB);
        }
      const u32 swz = (1u << a.tma_swizzle) - 1u;
      int k = 0;
      for (long long t = first; t < n_tiles; t += step, ++k) {
        const int st = k % STAGES;
        const u32 stage = stage0 + (u32)st * TILEB;
        const bool ok = mbar_wait_bounded(smem_u32(&tma_bar[g][st]), (u32)((k / STAGES) & 1));
        u64 ub[D];
#pragma unroll
        for (int j = 0; j < D / 2; ++j) {
          // this thread's row, 16 bytes at a time, at the tensor map's swizzled offsets
          const u32 off = (u32)(r * ROWB + 16 * j);
          const u32 addr = stage + (off ^ (((off >> 7) & swz) << 4));
          asm volatile("ld.shared.v2.u64 {%0, %1}, [%2];" : "=l"(ub[2 * j]), "=l"(ub[2 * j + 1]) : "r"(addr));
        }
        // one warp barrier both says the stage is read (it can be refilled
        // while the events are evaluated) and votes on the wait: if a copy
        // never completed, the rows just read are discarded and the warp
        // reports and stops
        const bool all_ok = __all_sync(0xffffffffu, ok);
        __syncwarp();
        if (!all_ok) {
          if (r == 0 && a.flags) atomicOr(a.flags, VF_FLAG_TIMEOUT);
          break;
        }
        if (r == 0 && t + STAGES * step < n_tiles) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          tma_load_tile(stage, a.tmap, 0, (int)((t + STAGES * step) * VF_INJ_ROWS), smem_u32(&tma_bar[g][st]),
                        TILEB);
        }
        const long long e = t * VF_INJ_ROWS + r;
        if (e < n) event(ub, e);
      }
    }
  }
  if (!tma) {
    const long long stride = (long long)gridDim.x * THREADS;
    const bool vec = (D % 2 == 0) && ((reinterpret_cast<size_t>(a.u_inj) & 15) == 0);
    for (long long e = (long long)blockIdx.x * THREADS + tid; e < n; e += stride) {
      const long long* up = reinterpret_cast<const long long*>(a.u_inj) + e * D;
      u64 ub[D];
      if (vec) {
#pragma unroll
        for (int j = 0; j < D / 2; ++j) {
          const longlong2 v = __ldcs(reinterpret_cast<const longlong2*>(up) + j);
          ub[2 * j] = (u64)v.x;
          ub[2 * j + 1] = (u64)v.y;
        }
      } else {
#pragma unroll
        for (int d = 0; d < D; ++d) ub[d] = (u64)__ldcs(up + d);
      }
      event(ub, e);
    }
  }
  if (bad && a.flags) atomicOr(a.flags, VF_FLAG_INDEX_RANGE);

  __shared__ double red[2][THREADS / 32];
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  if (lane == 0) {
    red[0][warp] = (double)s1.s + (double)s1.c;
    red[1][warp] = (double)s2.s + (double)s2.c;
  }
  __syncthreads();
  const int W = 2 + NB;
  double* row = a.partials + (long long)blockIdx.x * W;
  if (tid == 0) {
    double b1 = 0.0, b2 = 0.0;
    for (int i = 0; i < THREADS / 32; ++i) {
      b1 += red[0][i];
      b2 += red[1][i];
    }
    b1 *= wscale;
    b2 *= wscale * wscale;
    if ((!isfinite(b1) || !isfinite(b2)) && a.flags) atomicOr(a.flags, VF_FLAG_NONFINITE);
    if (a.accumulate) {
      row[0] += b1;
      row[1] += b2;
    } else {
      row[0] = b1;
      row[1] = b2;
    }
  }
  if (train) {
    const double s2c = wscale * wscale;
    for (int k = tid; k < NB; k += THREADS) {
      const int d = k / VF_BINS, b = k - d * VF_BINS;
      float hf = 0.0f;
      if (d < 2 * NP) {
        const float* tab = hist + (d >> 1) * 2500;
        if ((d & 1) == 0)
          for (int c = 0; c < VF_BINS; ++c) hf += tab[b * VF_BINS + c];  // row sum
        else
          for (int rr = 0; rr < VF_BINS; ++rr) hf += tab[rr * VF_BINS + b];  // column sum
      } else {
        hf = hist[NP * 2500 + b];
      }
      const double h = (double)hf * s2c;
      if (a.accumulate)
        row[2 + k] += h;
      else
        row[2 + k] = h;
    }
  }
  if (!a.accumulate)
    for (long long rr = blockIdx.x + (long long)gridDim.x; rr < a.rows_total; rr += gridDim.x)
      for (int k = tid; k < W; k += THREADS) a.partials[rr * W + k] = 0.0;
}

}  // namespace vf
