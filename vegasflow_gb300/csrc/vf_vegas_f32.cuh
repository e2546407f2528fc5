// The fused fp32 VEGAS sampler: the performance path of the float32 form.
//
// Compared with the generic sampler (vf_sample.cuh) this kernel is specialised
// at compile time on the exact dimension count and the integrand, draws the
// Philox words with round keys held in the parameter block, and stages a
// per-bin table that folds the importance map, the integration limits and --
// for the Gaussian family -- the integrand's affine argument into one fused
// multiply-add per dimension:
//
//   bin i, fraction m in [1, 2) from p = 50 * ~word + 25 (exact, 64-bit):
//       i = p >> 32,  m = 1 + (p mod 2^32) / 2^32  (23 bits)
//   table cell {c0, c1} per (dimension, bin), computed in float64 and rounded once:
//       generic integrand:  x  = c0 + c1 m,  c0 = xmin + (lo - delta) xdelta, c1 = delta xdelta
//       Gaussian family:    t  = c0 + c1 m,  t = (x - mu) sqrt(log2 e) / a,
//                           f  = 2^(-sum t^2)  (the normalisation goes to the float64 scale)
//   weight w = prod_d c1 (float32); the constant 50^D * xjac (* pref / prod k) is
//   applied in float64 to the block partials.
//
// Per event: accumulation of w f and (w f)^2 in TwoSum-compensated fp32, and
// (when training) the (w f)^2 histogram in shared memory, in one of three
// layouts (`hist_copies`; which is fastest depends on the dimension count and
// the spread of the weights, so the launch-shape autotuner chooses):
//   0      joint pairs (the default): dimensions (0,1), (2,3), ... share one
//          50 x 50 table per block, so an event makes ceil(D/2) float atomic
//          additions instead of D, and with 2500 cells the lanes of a warp rarely
//          collide on an address.  At the end each dimension's 50 bins are the
//          row or column sums of its pair's table (an odd last dimension keeps a
//          plain 50-bin table).
//   1,2,4  per-dimension tables, that many copies per warp (lane groups).
//   8      fixed point (VF_F32_HIST_FIXED): the joint pair tables of layout 0
//          as 32-bit integers, updated with native integer shared atomics (no
//          result read back) instead of float atomics, which the hardware runs
//          as compare-and-swap loops.  An event adds q = floor(S (w f)^2 + r),
//          r a per-event dither in [0, 1) (a Weyl sequence of the event number),
//          so the expectation of q / S is exact.  A cell cannot wrap: q is
//          capped at Qmax = (2^32 - 1) / (events the block walks), and an event
//          at or above the cap goes to a per-dimension float table instead.
//          Each block picks its power-of-two scale S from the first event of
//          every thread (S (w f)^2 about Qmax / 512 at their geometric mean);
//          a block whose first events are all zero uses the float table only.
//          The integer sums do not depend on the order of the atomics.
#pragma once
#include "vf_sample.cuh"

#ifndef VF_F32_MIN_BLOCKS
#define VF_F32_MIN_BLOCKS 4
#endif

namespace vf {

__device__ __forceinline__ float ex2_approx_ftz(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__host__ __device__ inline int vegas_f32_joint_floats(int D) { return (D / 2) * 2500 + (D & 1) * 50; }

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

// ---- TMA staging of injected uniforms (tiles of THREADS events x D float64)
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

// the fixed-point histogram layout (hist_copies value)
#define VF_F32_HIST_FIXED 8

__host__ __device__ inline int vegas_f32_smem_bytes(int D, int copies_per_warp, int train,
                                                    int threads = VF_THREADS) {
  const int nb = D * VF_BINS;
  int hist;
  if (copies_per_warp == 0)
    hist = vegas_f32_joint_floats(D) * 4;
  else if (copies_per_warp == VF_F32_HIST_FIXED)
    hist = (vegas_f32_joint_floats(D) + nb) * 4;  // integer joint tables, float overflow table
  else
    hist = (threads / 32) * copies_per_warp * nb * 4;
  return nb * 8 + (train ? hist : 0);
}

// THREADS: the block size (an autotuner choice, 128 or 256); the register cap
// (launch bounds) stays at 64 per thread for both.  TAP: the parity
// instantiation, which also writes every event's D bin indices to a.ind_out
// ([n_events][D] int32); the kernels of the hot path are TAP = false, where the
// writes do not exist.
template <int D, int INTEG, int THREADS = VF_THREADS, bool TAP = false>
__global__ void __launch_bounds__(THREADS, VF_F32_MIN_BLOCKS * VF_THREADS / THREADS)
vf_vegas_f32_kernel(const __grid_constant__ SampleArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NB = D * VF_BINS;
  constexpr bool GAUSS = (INTEG == VF_INT_SYMGAUSS || INTEG == VF_INT_GAUSS);
  float2* cells = reinterpret_cast<float2*>(smem);
  float* hist = reinterpret_cast<float*>(smem + NB * sizeof(float2));
  constexpr int NP = D / 2;  // joint pairs
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const bool train = a.train != 0;
  const bool limits = a.xmin != nullptr;
  const int cpw = a.hist_copies;
  const CallWords cw = call_words(a);
  const bool fixedp = train && cpw == VF_F32_HIST_FIXED;
  // fixed-point layout: integer joint tables (as layout 0), float overflow table [NB]
  u32* hint = reinterpret_cast<u32*>(hist);
  float* hovf = reinterpret_cast<float*>(hint + vegas_f32_joint_floats(D));

  // ---- per-block float64 constants: Gaussian centres and k_d = sqrt(log2 e)/a_d,
  // and the weight constant 50^D * xjac (* pref / prod k_d)
  __shared__ double g_mu[D], g_k[D], g_wscale;
  constexpr double SQRT_LOG2E = 1.2011224087864498;  // sqrt(log2(e))
  if (GAUSS && tid < D) {
    g_mu[tid] = (INTEG == VF_INT_SYMGAUSS) ? 0.5 : a.params[tid];
    g_k[tid] = SQRT_LOG2E / ((INTEG == VF_INT_SYMGAUSS) ? a.params[0] : a.params[D + tid]);
  }
  __syncthreads();
  if (tid == 0) {
    double ws = a.xjac;
    for (int d = 0; d < D; ++d) ws *= 50.0;
    if (GAUSS) {
      double prodk = 1.0;
      for (int d = 0; d < D; ++d) prodk *= g_k[d];
      ws *= ((INTEG == VF_INT_SYMGAUSS) ? a.params[1] : 1.0) / prodk;
    }
    g_wscale = ws;
  }

  // ---- stage the per-bin table (float64, rounded once) and clear the histograms
  for (int k = tid; k < NB; k += blockDim.x) {
    const int d = k / VF_BINS, b = k - d * VF_BINS;
    const double lo = a.grid[d * VF_EDGES + b];
    const double dl = a.grid[d * VF_EDGES + b + 1] - lo;
    double c0 = lo - dl, c1 = dl;
    if (limits) {
      c0 = a.xmin[d] + c0 * a.xdelta[d];
      c1 = c1 * a.xdelta[d];
    }
    if (GAUSS) {
      c0 = (c0 - g_mu[d]) * g_k[d];
      c1 = c1 * g_k[d];
    }
    cells[k] = make_float2((float)c0, (float)c1);
  }
  if (train) {
    if (cpw == 0)
      for (int k = tid; k < NP * 2500 + (D & 1) * VF_BINS; k += blockDim.x) hist[k] = 0.0f;
    else if (fixedp)
      for (int k = tid; k < vegas_f32_joint_floats(D) + NB; k += blockDim.x) hint[k] = 0u;  // 0 and 0.0f
    else
      for (int k = tid; k < (THREADS / 32) * cpw * NB; k += blockDim.x) hist[k] = 0.0f;
  }
  __syncthreads();

  // float64 constant of the weight (host-computed): 50^D * xjac, times
  // pref / prod k for the Gaussian family
  const double wscale = g_wscale;
  [[maybe_unused]] const float wscale_f = (float)wscale;  // the full weight handed to a user integrand
  IntegrandConsts<float, D> kc;
  if (!GAUSS) load_consts<D>(kc, INTEG == VF_INT_USER ? VF_INT_NONE : INTEG, a.params, D);

  float* my_hist = hist + (warp * cpw + ((lane * cpw) >> 5)) * NB;
  float hscale = 1.0f;  // fixed point: the block's power-of-two scale S
  float qcap = 0.0f;    // fixed point: Qmax (0: the float table only)
  F2 s1 = {0.0f, 0.0f}, s2 = {0.0f, 0.0f};

  // fixed point: add (w f)^2 of event `ev` to its D bins
  auto add_fixed = [&](const int (&bins)[D], float v2, u64 ev) {
    const float r = (float)((u32)ev * 0x9E3779B9u) * 2.3283064e-10f;  // Weyl dither in [0, 1)
    const float q = fmaf(v2, hscale, r);
    if (q < qcap) {
      const u32 qi = __float2uint_rd(q);
      if (qi != 0u) {
#pragma unroll
        for (int p = 0; p < NP; ++p)
          atomicAdd(hint + p * 2500 + (bins[2 * p] - 2 * p * VF_BINS) * VF_BINS +
                        (bins[2 * p + 1] - (2 * p + 1) * VF_BINS),
                    qi);
        if (D & 1) atomicAdd(hint + NP * 2500 + (bins[D - 1] - (D - 1) * VF_BINS), qi);
      }
    } else {
#pragma unroll
      for (int d = 0; d < D; ++d) atomicAdd(hovf + bins[d], v2);
    }
  };

  // one event from its per-dimension (bin, m) pairs; returns (w f)^2
  auto finish = [&](const int (&bins)[D], float wf, float s, const float (&x)[D]) -> float {
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
    if (train && !fixedp) {
      if (cpw == 0) {
#pragma unroll
        for (int p = 0; p < NP; ++p)
          atomicAdd(hist + p * 2500 + (bins[2 * p] - 2 * p * VF_BINS) * VF_BINS +
                        (bins[2 * p + 1] - (2 * p + 1) * VF_BINS),
                    v2);
        if (D & 1) atomicAdd(hist + NP * 2500 + (bins[D - 1] - (D - 1) * VF_BINS), v2);
      } else {
#pragma unroll
        for (int d = 0; d < D; ++d) atomicAdd(my_hist + bins[d], v2);
      }
    }
    return v2;
  };

  // parity tap: the event's bin indices (bins[] holds d 50 + bin)
  auto tap = [&](long long ev_idx, const int (&bins)[D]) {
    if constexpr (TAP) {
#pragma unroll
      for (int d = 0; d < D; ++d) a.ind_out[ev_idx * D + d] = bins[d] - d * VF_BINS;
    }
  };

  // one event's Philox words -> bins, weight and the Gaussian exponent (or x)
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
          const u64 pp = (u64)(~wq[j]) * 50ull + 25ull;
          const int i = (int)(pp >> 32);
          const float m = __uint_as_float(((u32)pp >> 9) | 0x3F800000u);
          const float2 c = cells[d * VF_BINS + i];
          const float t = fmaf(c.y, m, c.x);
          wf = (d == 0) ? c.y : wf * c.y;
          if (GAUSS)
            s = fmaf(t, t, s);
          else
            x[d] = t;
          bins[d] = d * VF_BINS + i;
        }
      }
    }
  };

  const long long n = a.n_events;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long e = (long long)blockIdx.x * blockDim.x + tid;
  if (a.u_inj == nullptr) {
    if (fixedp) {
      // Qmax from the most events the block walks, and the block's scale from
      // the first event of every thread: S = 2^k, k = floor(log2 Qmax) - 9 -
      // round(mean log2 (w f)^2) over the normal finite values
      __shared__ float lsum[THREADS / 32];
      __shared__ int lcnt[THREADS / 32];
      int bins[D];
      float x[D];
      float wf = 1.0f, s = 0.0f, v2 = 0.0f;
      const u64 ev = (u64)(a.ev_offset + e);
      const bool have = e < n;
      if (have) {
        draw(ev, bins, wf, s, x);
        v2 = finish(bins, wf, s, x);
        tap(e, bins);
      }
      const bool use = have && v2 >= 1.17549435e-38f && v2 <= 3.40282347e38f;  // normal, finite
      float l = use ? __log2f(v2) : 0.0f;
      int c = use ? 1 : 0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        l += __shfl_xor_sync(0xffffffffu, l, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
      }
      if (lane == 0) {
        lsum[warp] = l;
        lcnt[warp] = c;
      }
      __syncthreads();
      float ls = 0.0f;
      int cs = 0;
#pragma unroll
      for (int i = 0; i < THREADS / 32; ++i) {
        ls += lsum[i];
        cs += lcnt[i];
      }
      const long long per_thread = n > 0 ? (n + stride - 1) / stride : 1;
      const float cap = floorf((float)(4294967295.0 / ((double)THREADS * (double)per_thread)));
      const int cap_log2 = (int)((__float_as_uint(cap) >> 23) & 0xFF) - 127;  // floor(log2 Qmax)
      int k = cap_log2 - 9 - (cs > 0 ? __float2int_rn(ls / (float)cs) : 0);
      k = k < -126 ? -126 : (k > 127 ? 127 : k);
      hscale = __int_as_float((127 + k) << 23);  // 2^k
      qcap = cs > 0 ? cap : 0.0f;
      if (have) add_fixed(bins, v2, ev);
      e += stride;
    }
    // Two events per pass give the scheduler two independent draws to overlap
    // (shared-memory latency of one with the Philox rounds of the other).
    // Measured (1e8 events): faster for D <= 4 (0.560 vs 0.582 ms training,
    // 0.441 vs 0.490 frozen).  For D >= 5 it made frozen grids faster too (D = 8:
    // 0.717 vs 0.799 ms) but training slower (D = 8: 0.984 vs 0.975 ms, the
    // histogram atomics dominate), and the registers it needs slow the training
    // loop even where it is not taken, so it is compiled for D <= 4 only.
    if constexpr (D <= 4) if (!fixedp) {
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
      const u64 ev = (u64)(a.ev_offset + e);
      int bins[D];
      float x[D];
      float wf = 1.0f, s = 0.0f;
      draw(ev, bins, wf, s, x);
      const float v2 = finish(bins, wf, s, x);
      if (fixedp) add_fixed(bins, v2, ev);
      tap(e, bins);
    }
  } else {
    // injected float64 uniforms, [n][D] row-major, streamed once
    int bad = 0;
    auto injected_event = [&](const u64 (&ub)[D], long long ev_idx) {
      int bins[D];
      float x[D];
      float wf = 1.0f, s = 0.0f;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        int i;
        float m;
        if (!inj_bin_exact(ub[d], i, m)) {
          // the bin in float64, bit-exact with the reference (vflow.py:117, :67)
          const double xn = __dmul_rn(50.0, __dsub_rn(1.0, __longlong_as_double((long long)ub[d])));
          i = (int)xn;
          if (i < 0 || i > VF_BINS - 1) {
            bad = 1;
            i = i < 0 ? 0 : VF_BINS - 1;
          }
          m = (float)(1.0 + (xn - floor(xn)));
        }
        const float2 c = cells[d * VF_BINS + i];
        const float t = fmaf(c.y, m, c.x);
        wf = (d == 0) ? c.y : wf * c.y;
        if (GAUSS)
          s = fmaf(t, t, s);
        else
          x[d] = t;
        bins[d] = d * VF_BINS + i;
      }
      const float v2 = finish(bins, wf, s, x);
      if (fixedp)  // injected uniforms: the float table, no scale
        for (int d = 0; d < D; ++d) atomicAdd(hovf + bins[d], v2);
      tap(ev_idx, bins);
    };
    if (a.tma_swizzle != 0 && (D == 4 || D == 8 || D == 16)) {
      // Tiles of THREADS events (the grid-stride assignment: tile t holds
      // events t THREADS .. t THREADS + THREADS - 1, thread i takes event i)
      // brought in by TMA into one shared-memory stage; the tensor map's
      // swizzle (32/64/128 bytes for rows of 32/64/128 bytes) makes every
      // quarter-warp read of a row conflict-free.  Each thread copies its row to
      // registers, the block syncs, the next tile's copy is issued and then the
      // events are evaluated, so the copy overlaps the arithmetic with a
      // single 8 D THREADS-byte stage (registers are the second buffer).
      constexpr int ROWB = 8 * D;
      constexpr u32 TILEB = THREADS * ROWB;  // a multiple of 1024
      __shared__ alignas(8) u64 tma_bar;
      const u32 stage =
          (smem_u32(smem) + (u32)vegas_f32_smem_bytes(D, cpw, a.train, THREADS) + 1023u) & ~1023u;
      const u32 bar = smem_u32(&tma_bar);
      const long long n_tiles = (n + THREADS - 1) / THREADS;
      const long long G = gridDim.x;
      if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (blockIdx.x < n_tiles) tma_load_tile(stage, a.tmap, 0, (int)(blockIdx.x * THREADS), bar, TILEB);
      }
      __syncthreads();
      const u32 swz = (1u << a.tma_swizzle) - 1u;
      u32 parity = 0;
      for (long long t = blockIdx.x; t < n_tiles; t += G) {
        const bool ok = mbar_wait_bounded(bar, parity);
        parity ^= 1u;
        if (!__syncthreads_and(ok)) {  // a copy never completed: report, stop
          if (tid == 0 && a.flags) atomicOr(a.flags, VF_FLAG_TIMEOUT);
          break;
        }
        u64 ub[D];
#pragma unroll
        for (int j = 0; j < D / 2; ++j) {
          const u32 off = (u32)(tid * ROWB + 16 * j);
          const u32 addr = stage + (off ^ (((off >> 7) & swz) << 4));
          asm volatile("ld.shared.v2.u64 {%0, %1}, [%2];" : "=l"(ub[2 * j]), "=l"(ub[2 * j + 1]) : "r"(addr));
        }
        __syncthreads();  // the stage is read: refill it while the events are evaluated
        if (tid == 0 && t + G < n_tiles) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          tma_load_tile(stage, a.tmap, 0, (int)((t + G) * THREADS), bar, TILEB);
        }
        if (t * THREADS + tid < n) injected_event(ub, t * THREADS + tid);
      }
    } else {
      // plain loads: 16-byte (evict-first) when D is even and the array is
      // 16-byte aligned
      const bool vec = (D % 2 == 0) && ((reinterpret_cast<size_t>(a.u_inj) & 15) == 0);
      for (; e < n; e += stride) {
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
        injected_event(ub, e);
      }
    }
    if (bad && a.flags) atomicOr(a.flags, VF_FLAG_INDEX_RANGE);
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
    // marginals / copy sums in fp32 (the tables are fp32), one float64 scaling per bin
    const double s2c = wscale * wscale;
    const int ncopies = (THREADS / 32) * cpw;
    for (int k = tid; k < NB; k += blockDim.x) {
      float hf = 0.0f;
      if (cpw == 0) {
        const int d = k / VF_BINS, b = k - d * VF_BINS;
        if (d < 2 * NP) {
          const float* tab = hist + (d >> 1) * 2500;
          if ((d & 1) == 0)
            for (int c = 0; c < VF_BINS; ++c) hf += tab[b * VF_BINS + c];  // row sum
          else
            for (int r = 0; r < VF_BINS; ++r) hf += tab[r * VF_BINS + b];  // column sum
        } else {
          hf = hist[NP * 2500 + b];
        }
      } else if (fixedp) {
        const int d = k / VF_BINS, b = k - d * VF_BINS;
        u64 total = 0;
        if (d < 2 * NP) {
          const u32* tab = hint + (d >> 1) * 2500;
          if ((d & 1) == 0)
            for (int c = 0; c < VF_BINS; ++c) total += tab[b * VF_BINS + c];  // row sum
          else
            for (int r = 0; r < VF_BINS; ++r) total += tab[r * VF_BINS + b];  // column sum
        } else {
          total = hint[NP * 2500 + b];
        }
        hf = hovf[k];
        const double h = ((double)total / (double)hscale + (double)hf) * s2c;
        if (a.accumulate)
          row[2 + k] += h;
        else
          row[2 + k] = h;
        continue;
      } else {
        for (int c = 0; c < ncopies; ++c) hf += hist[c * NB + k];
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
      for (int k = tid; k < W; k += blockDim.x) a.partials[r * W + k] = 0.0;
}

}  // namespace vf
