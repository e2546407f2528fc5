// Batched VEGAS: many independent integrals (own dimension count, event count,
// integrand, grid) in one persistent fp32 launch per iteration.
//
// Work unit: a tile = a contiguous range of at most `tile_events` events of one
// integral, tile boundaries at fixed multiples within the integral.  A tile's
// result depends only on the integral and the tile (Philox counter = event index
// within the integral, stream id = the integral's own id), never on which block
// ran it or on the other integrals of the batch: an integral gives the same
// result alone and in any mix (up to the histogram's float atomics order).
//
// Per-integral state lives in slots (iteration index, Philox call counter,
// history, running average), so integrals can join and leave a batch between
// iterations (continuous batching) while keeping their own progress.
//
// A user integrand (CUDA source, NVRTC) gets its own build of the sampler with
// the device function inlined (USER = true): the integrals of one launch then
// all use that function, each with its own parameters.
//
// The sampler is persistent: each block takes tiles from a device queue (an
// atomic counter), stages the tile's integral (per-bin table, constants) in
// shared memory when it differs from the previous tile, processes the tile with
// the same specialised code as the single-integral fp32 kernel, and writes the
// tile's partial row [res, res2, hist[D][50]] (float64).  The batched
// iteration-end kernel then sums each integral's tile rows in tile order.
#pragma once
#include "vf_vegas_f32.cuh"

namespace vf {

// One integral of a batch (mirrors vf_batch_item in include/vegasflow_gb300.h).
struct BatchItem {
  long long n_events;
  long long grid_off;   // doubles into `grids` ([n_dim][51])
  long long param_off;  // doubles into `params`
  double xjac;          // 1 / n_events
  int n_dim;
  int integrand;        // VF_INT_SYMGAUSS .. VF_INT_SUM, or a vf_jit_integrand id (VF_ALG_BATCH)
  int stream_id;        // Philox counter word 3: independent stream per integral
  int tile0;            // first tile
  int n_tiles;
  int train;
  int slot;             // state slot: iters[slot], calls[slot], history[slot], avg[slot]
  int pad;
};

struct BatchArgs {
  const BatchItem* items;
  const int* tile_item;        // [n_tiles]
  const long long* tile_start; // [n_tiles] first event of the tile within its integral
  const int* tile_count;       // [n_tiles]
  const long long* tile_row;   // [n_tiles] offset (doubles) of the tile's partial row
  int* queue;                  // work counter, zero at launch
  const unsigned int* calls;   // [slots] Philox call counter of each integral's iteration
  const double* grids;
  const double* params;
  double* partials;
  int* flags;
  int n_tiles;
  int max_dim;
  RoundKeys rk;
};

__host__ __device__ inline int batch_smem_bytes(int max_dim) {
  return max_dim * VF_BINS * 8 + vegas_f32_joint_floats(max_dim) * 4;
}

// Stage one integral (table cells, weight constant) in shared memory; the
// cells' binary exponents go into *expsum (zeroed by the caller before this
// function's first barrier) for the weight prescale (f32_prescale_exponent).
template <int D, bool GAUSS>
__device__ __forceinline__ double batch_stage(const BatchItem& it, const double* __restrict__ grids,
                                              const double* __restrict__ params, float2* cells,
                                              double* g_mu, double* g_k, int* expsum) {
  constexpr double SQRT_LOG2E = 1.2011224087864498;
  const double* grid = grids + it.grid_off;
  const double* p = params + it.param_off;
  const int tid = threadIdx.x;
  if (GAUSS && tid < D) {
    g_mu[tid] = it.integrand == VF_INT_SYMGAUSS ? 0.5 : p[tid];
    g_k[tid] = SQRT_LOG2E / (it.integrand == VF_INT_SYMGAUSS ? p[0] : p[D + tid]);
  }
  __syncthreads();
  int mine = 0;
  for (int k = tid; k < D * VF_BINS; k += blockDim.x) {
    const int d = k / VF_BINS, b = k - d * VF_BINS;
    const double lo = grid[d * VF_EDGES + b];
    const double dl = grid[d * VF_EDGES + b + 1] - lo;
    double c0 = lo - dl, c1 = dl;
    if (GAUSS) {
      c0 = (c0 - g_mu[d]) * g_k[d];
      c1 = c1 * g_k[d];
    }
    mine += f32_cell_exponent(c1);
    cells[k] = make_float2((float)c0, (float)c1);
  }
  f32_add_exponents(expsum, mine);
  double ws = it.xjac;
  for (int d = 0; d < D; ++d) ws *= 50.0;
  if (GAUSS) {
    double prodk = 1.0;
    for (int d = 0; d < D; ++d) prodk *= g_k[d];
    ws *= (it.integrand == VF_INT_SYMGAUSS ? p[1] : 1.0) / prodk;
  }
  return ws;
}

// Process one tile of an integral with D dimensions (USER: the integrand is
// the program's VF_USER_FN).
template <int D, bool GAUSS, bool USER>
__device__ void batch_tile(const BatchArgs& a, const BatchItem& it, int tile, bool restage,
                           unsigned char* smem, double* g_mu, double* g_k, double* s_wscale) {
  constexpr int NB = D * VF_BINS;
  constexpr int NP = D / 2;
  float2* cells = reinterpret_cast<float2*>(smem);
  float* hist = reinterpret_cast<float*>(smem + a.max_dim * VF_BINS * 8);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool train = it.train != 0;
  __shared__ int s_expsum;  // the staged integral's cell exponents (kept until the next restage)
  if (restage) {
    if (tid == 0) s_expsum = 0;
    const double ws = batch_stage<D, GAUSS>(it, a.grids, a.params, cells, g_mu, g_k, &s_expsum);
    if (tid == 0) *s_wscale = ws;
  }
  if (train)
    for (int k = tid; k < NP * 2500 + (D & 1) * VF_BINS; k += blockDim.x) hist[k] = 0.0f;
  __syncthreads();
  // the weight prescale 2^kw of the fp32 samplers (exact; the float64 scale takes it back)
  const int kw = f32_prescale_exponent(s_expsum);
  const float wpre = __int_as_float((127 + kw) << 23);
  const double wscale = *s_wscale * ldexp(1.0, -kw);
  const float wscale_f = (float)wscale;  // the full weight handed to a user integrand
  const double* iparams = a.params + it.param_off;
  IntegrandConsts<float, D> kc;
  if (!GAUSS && !USER) load_consts<D>(kc, it.integrand, iparams, D);
  const u32 call = a.calls[it.slot];
  const u32 c3 = (u32)it.stream_id;
  F2 s1 = {0.0f, 0.0f}, s2 = {0.0f, 0.0f};
  const long long start = a.tile_start[tile];
  const int count = a.tile_count[tile];
  for (int j = tid; j < count; j += blockDim.x) {
    const u64 ev = (u64)(start + j);
    int bins[D];
    float x[D];
    float wf = 1.0f, s = 0.0f;
#pragma unroll
    for (int q = 0; q < (D + 3) / 4; ++q) {
      u32 c0 = (u32)ev, c1 = (u32)(ev >> 32), c2 = (call << 4) | (u32)q, cc3 = c3;
      philox4x32_10_rk(c0, c1, c2, cc3, a.rk);
      const u32 wq[4] = {c0, c1, c2, cc3};
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        const int d = 4 * q + jj;
        if (d < D) {
          const u64 pp = (u64)(~wq[jj]) * 50ull + 25ull;
          const int i = (int)(pp >> 32);
          const float m = __uint_as_float(((u32)pp >> 9) | 0x3F800000u);
          const float2 c = cells[d * VF_BINS + i];
          const float t = fmaf(c.y, m, c.x);
          wf = (d == 0) ? wpre * c.y : wf * c.y;
          if (GAUSS)
            s = fmaf(t, t, s);
          else
            x[d] = t;
          bins[d] = i;
        }
      }
    }
    float f;
    if constexpr (GAUSS) {
      f = ex2_approx_ftz(-s);
    } else if constexpr (USER) {
#ifdef VF_JIT_USER
      f = (float)VF_USER_FN(x, D, wf * wscale_f, iparams);
#else
      f = 0.0f;  // a user build always defines VF_JIT_USER
#endif
    } else {
      f = eval_builtin<D>(it.integrand, x, D, kc);
    }
    const float v = wf * f;
    const float v2 = v * v;
    two_sum_add(s1, v);
    two_sum_add(s2, v2);
    if (train) {
#pragma unroll
      for (int pq = 0; pq < NP; ++pq) atomicAdd(hist + pq * 2500 + bins[2 * pq] * VF_BINS + bins[2 * pq + 1], v2);
      if (D & 1) atomicAdd(hist + NP * 2500 + bins[D - 1], v2);
    }
  }
  __shared__ double red[2][VF_THREADS / 32];
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  if (lane == 0) {
    red[0][warp] = (double)s1.s + (double)s1.c;
    red[1][warp] = (double)s2.s + (double)s2.c;
  }
  __syncthreads();
  double* row = a.partials + a.tile_row[tile];
  if (tid == 0) {
    double b1 = 0.0, b2 = 0.0;
    for (int i = 0; i < VF_THREADS / 32; ++i) {
      b1 += red[0][i];
      b2 += red[1][i];
    }
    row[0] = b1 * wscale;
    row[1] = b2 * wscale * wscale;
  }
  if (train) {
    const double s2c = wscale * wscale;
    for (int k = tid; k < NB; k += blockDim.x) {
      const int d = k / VF_BINS, b = k - d * VF_BINS;
      float hf = 0.0f;
      if (d < 2 * NP) {
        const float* tab = hist + (d >> 1) * 2500;
        if ((d & 1) == 0)
          for (int c = 0; c < VF_BINS; ++c) hf += tab[b * VF_BINS + c];
        else
          for (int r = 0; r < VF_BINS; ++r) hf += tab[r * VF_BINS + b];
      } else {
        hf = hist[NP * 2500 + b];
      }
      row[2 + k] = (double)hf * s2c;
    }
  }
  __syncthreads();  // the shared tables are reused by the next tile
}

template <bool GAUSS, int DC, bool USER>
__device__ __forceinline__ void batch_dispatch(int D, const BatchArgs& a, const BatchItem& it, int tile,
                                               bool restage, unsigned char* smem, double* g_mu,
                                               double* g_k, double* s_ws) {
  switch (D) {
#define VF_BATCH_CASE(n) \
  case n: \
    if constexpr (n <= DC) batch_tile<n, GAUSS, USER>(a, it, tile, restage, smem, g_mu, g_k, s_ws); \
    break;
    VF_BATCH_CASE(1) VF_BATCH_CASE(2) VF_BATCH_CASE(3) VF_BATCH_CASE(4) VF_BATCH_CASE(5)
    VF_BATCH_CASE(6) VF_BATCH_CASE(7) VF_BATCH_CASE(8) VF_BATCH_CASE(9) VF_BATCH_CASE(10)
    VF_BATCH_CASE(11) VF_BATCH_CASE(12) VF_BATCH_CASE(13) VF_BATCH_CASE(14) VF_BATCH_CASE(15)
    VF_BATCH_CASE(16)
#undef VF_BATCH_CASE
    default: break;
  }
}

// USER: the build for a user integrand (every integral of the launch uses it).
// DC: the dimension class of the launch (8: every integral has n_dim <= 8, its
// joint tables fit four blocks per SM; 16: any n_dim, two blocks per SM).
// (Measured on the 1,024-integral batch: four blocks per SM with a few spilled
// registers beat three without: 18.96 vs 19.15 ms per iteration.)  The
// host launches one sampler per class present, each over its own tiles.
template <int DC, bool USER = false>
__global__ void __launch_bounds__(VF_THREADS, DC <= 8 ? 4 : 2) vf_batch_sample_kernel(const BatchArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double g_mu[VF_MAX_DIM], g_k[VF_MAX_DIM], s_ws;
  __shared__ int s_tile;
  int cur_item = -1;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(a.queue, 1);
    __syncthreads();
    const int tile = s_tile;
    __syncthreads();
    if (tile >= a.n_tiles) break;
    const int item = a.tile_item[tile];
    const BatchItem it = a.items[item];
    const bool restage = item != cur_item;
    cur_item = item;
    if constexpr (USER)
      batch_dispatch<false, DC, true>(it.n_dim, a, it, tile, restage, smem, g_mu, g_k, &s_ws);
    else if (it.integrand == VF_INT_SYMGAUSS || it.integrand == VF_INT_GAUSS)
      batch_dispatch<true, DC, false>(it.n_dim, a, it, tile, restage, smem, g_mu, g_k, &s_ws);
    else
      batch_dispatch<false, DC, false>(it.n_dim, a, it, tile, restage, smem, g_mu, g_k, &s_ws);
  }
}

}  // namespace vf
