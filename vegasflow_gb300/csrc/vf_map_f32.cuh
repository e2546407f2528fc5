// The fp32 VEGAS map without an integrand: the sampler API
// (generate_random_array, monte_carlo.py:229-275; vflow.py:93-126) and the
// sampling half of a torch-evaluated iteration.  Per event the same draw as the
// fused Philox sampler -- ceil(D/4) Philox blocks, the exact integer map on
// p = 50 w + 25 through the reversed, lane-replicated per-bin table {C0, C1}
// (vf_vegas_f32.cuh) -- and the event's x (D floats), weight w (float) and,
// when asked (IND), reference bin indices (D int32) go to HBM.
//
// The stores are most of the cost (36 bytes per event at D = 8 for x and w), so
// they are staged: each warp writes its lanes' rows into its own shared-memory
// tile of 32 EPT events and lane 0 hands each full tile to the bulk-copy engine
// (cp.async.bulk shared -> global, contiguous, 16-byte aligned), with
// `map_tiles` tiles per warp in flight and no block-wide barrier.  A thread's
// own row stores would cost a warp 32 separate 32-byte segments per dimension;
// a tile is one contiguous transfer.  The last partial tile, and arrays that
// are not 16-byte aligned, use plain stores.  1024 threads per block, one block
// per SM; each lane draws up to 4 events per tile (independent Philox chains,
// and the per-tile hand-off paid once for all of them), and where shared
// memory allows each warp has two tiles in flight and the table 16
// lane-replicated copies (conflict-free lookups): map_shape.
#pragma once
#include "vf_vegas_f32.cuh"

namespace vf {

#define VF_MAP_THREADS 1024
#ifndef VF_MAP_EPT_MAX
#define VF_MAP_EPT_MAX 4  // events per lane per warp tile, at most
#endif
#ifndef VF_MAP_TILES_MAX
#define VF_MAP_TILES_MAX 2  // tiles per warp in flight, at most
#endif
#ifndef VF_MAP_TC_MAX
#define VF_MAP_TC_MAX 16  // lane-replicated table copies, at most
#endif

// Bytes of one warp tile of 32 ept events [x: D floats][ind: D ints][w: 1 float]
// per event.
__host__ __device__ constexpr int map_tile_bytes(int D, bool ind, int ept) {
  return 32 * ept * (4 * D * (ind ? 2 : 1) + 4);
}
__host__ __device__ constexpr bool map_fit(int D, bool ind, int tc, int ept, int tiles) {
  return D * VF_BINS * tc * 8 + 16 + (VF_MAP_THREADS / 32) * tiles * map_tile_bytes(D, ind, ept) <= VF_SMEM_LIMIT;
}
// The kernel's shape for (D, ind), packed as tc * 100 + ept * 10 + tiles: the
// first of (4, 3, 2, 1 events per lane) x (2 tiles per warp in flight, then 1)
// x (16 table copies, then 1) that fits in shared memory.  Measured at D = 8
// (1e8 events): 1 event per lane 0.97 ms, 2: 0.83 ms, 3 to 6: 0.785-0.795 ms;
// tiles in flight and table copies move it by 1 % at most.
__host__ __device__ constexpr int map_shape(int D, bool ind) {
  for (int ept = VF_MAP_EPT_MAX; ept >= 1; --ept)
    for (int tiles = VF_MAP_TILES_MAX; tiles >= 1; --tiles)
      for (int tc = VF_MAP_TC_MAX; tc >= 1; tc = tc > 1 ? 1 : 0)
        if (map_fit(D, ind, tc, ept, tiles)) return tc * 100 + ept * 10 + tiles;
  return 0;
}
__host__ __device__ constexpr int map_tc(int D, bool ind) { return map_shape(D, ind) / 100; }
__host__ __device__ constexpr int map_ept(int D, bool ind) { return map_shape(D, ind) / 10 % 10; }
__host__ __device__ constexpr int map_tiles(int D, bool ind) { return map_shape(D, ind) % 10; }

__host__ __device__ inline int vegas_f32_map_smem_bytes(int D, bool ind) {
  return D * VF_BINS * map_tc(D, ind) * 8 + 16 +
         (VF_MAP_THREADS / 32) * map_tiles(D, ind) * map_tile_bytes(D, ind, map_ept(D, ind));
}

// One event's row of D 32-bit words into the staging tile in 16-byte stores (D a
// multiple of 4), 8-byte stores (D even) or word stores (D odd: conflict-free).
// Rows are 4 D bytes apart, so a warp storing word by word puts gcd(D, 32) lanes
// on one bank (8 at D = 8); a 16-byte store is served per quarter-warp, whose 8
// lanes then share a bank at most D / 4 ways (2 at D = 8).
template <int D>
__device__ __forceinline__ void stage_row(u32* dst, const u32 (&v)[D]) {
  if constexpr (D % 4 == 0) {
#pragma unroll
    for (int q = 0; q < D / 4; ++q)
      reinterpret_cast<uint4*>(dst)[q] = make_uint4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  } else if constexpr (D % 2 == 0) {
#pragma unroll
    for (int q = 0; q < D / 2; ++q) reinterpret_cast<uint2*>(dst)[q] = make_uint2(v[2 * q], v[2 * q + 1]);
  } else {
#pragma unroll
    for (int d = 0; d < D; ++d) dst[d] = v[d];
  }
}

__device__ __forceinline__ void bulk_store(void* gdst, u32 ssrc, u32 bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(ssrc), "r"(bytes)
               : "memory");
}

// Wait until at most N of this thread's bulk-copy groups still read shared memory.
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}

template <int D, bool IND>
__global__ void __launch_bounds__(VF_MAP_THREADS, 1) vf_vegas_f32_map_kernel(const __grid_constant__ SampleArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NB = D * VF_BINS;
  constexpr int TC = map_tc(D, IND);
  constexpr int EPT = map_ept(D, IND);
  constexpr int NT = map_tiles(D, IND);
  static_assert(TC >= 1 && EPT >= 1 && NT >= 1, "no map kernel shape fits in shared memory");
  constexpr int DSTRIDE = VF_BINS * TC * 8;
  float2* cells = reinterpret_cast<float2*>(smem);
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const CallWords cw = call_words(a);
  float* x_out = static_cast<float*>(a.x_out);
  float* w_out = static_cast<float*>(a.w_out);
  int* ind_out = a.ind_out;

  // ---- the weight constant 50^D xjac (-1)^D, and the reversed, replicated
  // per-bin table (x = c0 + c1 (1 + frac), c0 = xmin + (lo - delta) xdelta,
  // c1 = delta xdelta; cell j holds bin 49 - j as C0 = c0 + 3 c1, C1 = -c1)
  __shared__ double g_wscale;
  __shared__ int g_expsum;
  if (tid == 0) {
    double ws = (D & 1) ? -a.xjac : a.xjac;
    for (int d = 0; d < D; ++d) ws *= 50.0;
    g_wscale = ws;
    g_expsum = 0;
  }
  __syncthreads();  // g_expsum zeroed before the warps add to it
  int expsum = 0;
  for (int k = tid; k < NB; k += VF_MAP_THREADS) {
    const int d = k / VF_BINS, b = k - d * VF_BINS;
    const double lo = a.grid[d * VF_EDGES + b];
    const double dl = a.grid[d * VF_EDGES + b + 1] - lo;
    double c0 = lo - dl, c1 = dl;
    if (a.xmin != nullptr) {
      c0 = __fma_rn(c0, a.xdelta[d], a.xmin[d]);
      c1 = c1 * a.xdelta[d];
    }
    expsum += f32_cell_exponent(c1);
    const float2 cell = make_float2((float)__fma_rn(3.0, c1, c0), (float)(-c1));
    float2* dst = cells + (d * VF_BINS + (VF_BINS - 1 - b)) * TC;
#pragma unroll
    for (int c = 0; c < TC; ++c) dst[c] = cell;
  }
  f32_add_exponents(&g_expsum, expsum);
  __syncthreads();
  // the running product starts at 2^kw (no float32 underflow of prod_d c1 at
  // large D); the float constant takes 2^-kw back
  const int kw = f32_prescale_exponent(g_expsum);
  const float wpre = __int_as_float((127 + kw) << 23);
  const float wscale = (float)(g_wscale * ldexp(1.0, -kw));
  const char* mytab = reinterpret_cast<const char*>(cells + (lane & (TC - 1)));

  // ---- staging: per warp NT tiles of WT = 32 EPT events
  unsigned char* stage0 = smem + ((NB * TC * 8 + 15) & ~15);
  const bool aligned = ((reinterpret_cast<size_t>(x_out) | reinterpret_cast<size_t>(w_out) |
                         reinterpret_cast<size_t>(ind_out)) & 15) == 0;
  const long long n = a.n_events;
  constexpr int WT = 32 * EPT;
  constexpr u32 XBW = WT * D * 4, WBW = WT * 4;
  constexpr u32 TILEB = map_tile_bytes(D, IND, EPT);
  unsigned char* wbase = stage0 + (size_t)warp * NT * TILEB;
  const long long n_wt = (n + WT - 1) / WT;
  int it = 0;
  for (long long t = (long long)blockIdx.x * (VF_MAP_THREADS / 32) + warp; t < n_wt;
       t += (long long)gridDim.x * (VF_MAP_THREADS / 32), ++it) {
    const long long e0 = t * WT;
    const bool full = aligned && e0 + WT <= n;  // warp-uniform
    unsigned char* st = wbase + (it % NT) * TILEB;
    u32* xs = reinterpret_cast<u32*>(st);
    u32* is = reinterpret_cast<u32*>(st + XBW);
    float* wsm = reinterpret_cast<float*>(st + XBW * (IND ? 2 : 1));
    if (full) {
      // the stage's previous tile (NT tiles back) must have been read out
      if (lane == 0) bulk_wait_read<NT - 1>();
      __syncwarp();
    }
#pragma unroll
    for (int k = 0; k < EPT; ++k) {
      const int r = k * 32 + lane;  // row in the warp's tile
      const long long e = e0 + r;
      if (e < n) {
        const u64 ev = (u64)(a.ev_offset + e);
        float wf;
        u32 xr[D];  // x as float bits
        u32 br[D];
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
              // 1 + the top 23 bits of the low word as a float (no carry: < 2^23)
              const float m = __uint_as_float(((u32)pp >> 9) + 0x3F800000u);
              const float2 c = *reinterpret_cast<const float2*>(mytab + jj * (TC * 8) + d * DSTRIDE);
              xr[d] = __float_as_uint(fmaf(c.y, m, c.x));
              wf = (d == 0) ? wpre * c.y : wf * c.y;
              br[d] = (u32)(VF_BINS - 1) - jj;
            }
          }
        }
        const float w = wf * wscale;
        if (full) {
          stage_row<D>(xs + r * D, xr);
          if (IND) stage_row<D>(is + r * D, br);
          wsm[r] = w;
        } else {
          if (x_out)
#pragma unroll
            for (int d = 0; d < D; ++d) x_out[e * D + d] = __uint_as_float(xr[d]);
          if (IND)
#pragma unroll
            for (int d = 0; d < D; ++d) ind_out[e * D + d] = (int)br[d];
          if (w_out) w_out[e] = w;
        }
      }
    }
    if (full) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the rows, to the copy engine
      __syncwarp();
      if (lane == 0) {
        if (x_out) bulk_store(x_out + e0 * D, smem_u32(xs), XBW);
        if (IND) bulk_store(ind_out + e0 * D, smem_u32(is), XBW);
        if (w_out) bulk_store(w_out + e0, smem_u32(wsm), WBW);
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      }
    }
  }
  if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

}  // namespace vf
