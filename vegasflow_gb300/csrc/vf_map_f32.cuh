// The fp32 VEGAS map without an integrand: the sampler API
// (generate_random_array, monte_carlo.py:229-275; vflow.py:93-126) and the
// sampling half of a torch-evaluated iteration.  Per event the same draw as the
// fused sampler -- ceil(D/4) Philox blocks, the exact integer bin/fraction map,
// one FMA through the staged per-bin table -- and the event's x (D floats),
// weight w (float) and, when asked, bin indices (D int32) go to HBM.
//
// The stores are most of the cost (36 bytes per event at D = 8 for x and w), so
// they are staged: each warp writes its lanes' rows into its own shared-memory
// tile of VF_MAP_EPT x 32 events, and lane 0 hands each full tile to the
// bulk-copy engine (cp.async.bulk shared -> global, contiguous, 16-byte
// aligned), two tiles per warp in flight, with no block-wide barrier (measured
// 2 % faster than block tiles behind __syncthreads).  A thread's own row stores
// would cost a warp 32 separate 32-byte segments per dimension; a tile is one
// contiguous transfer.  The last partial tile, and arrays that are not 16-byte
// aligned, use plain stores.
#pragma once
#include "vf_vegas_f32.cuh"

namespace vf {

// events per thread per tile
#define VF_MAP_EPT 2

// resident blocks per SM the register allocation is sized for (256 threads)
#ifndef VF_MAP_MIN_BLOCKS
#define VF_MAP_MIN_BLOCKS 4
#endif

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

__host__ __device__ inline int vegas_f32_map_smem_bytes(int D, int threads, bool with_ind) {
  const int stage = VF_MAP_EPT * threads * (D * 4 * (with_ind ? 2 : 1) + 4);
  return D * VF_BINS * 8 + 2 * stage + 128;
}

__device__ __forceinline__ void bulk_store(void* gdst, u32 ssrc, u32 bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(ssrc), "r"(bytes)
               : "memory");
}

template <int D, int THREADS = VF_THREADS>
__global__ void __launch_bounds__(THREADS, VF_MAP_MIN_BLOCKS * VF_THREADS / THREADS)
vf_vegas_f32_map_kernel(const __grid_constant__ SampleArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NB = D * VF_BINS;
  float2* cells = reinterpret_cast<float2*>(smem);
  const int tid = threadIdx.x;
  const bool limits = a.xmin != nullptr;
  const CallWords cw = call_words(a);
  float* x_out = static_cast<float*>(a.x_out);
  float* w_out = static_cast<float*>(a.w_out);
  int* ind_out = a.ind_out;

  // ---- the weight constant 50^D * xjac, and the per-bin table {c0, c1}:
  // x = c0 + c1 m, c0 = xmin + (lo - delta) xdelta, c1 = delta xdelta
  __shared__ float g_wscale;
  if (tid == 0) {
    double ws = a.xjac;
    for (int d = 0; d < D; ++d) ws *= 50.0;
    g_wscale = (float)ws;
  }
  for (int k = tid; k < NB; k += blockDim.x) {
    const int d = k / VF_BINS, b = k - d * VF_BINS;
    const double lo = a.grid[d * VF_EDGES + b];
    const double dl = a.grid[d * VF_EDGES + b + 1] - lo;
    double c0 = lo - dl, c1 = dl;
    if (limits) {
      c0 = a.xmin[d] + c0 * a.xdelta[d];
      c1 = c1 * a.xdelta[d];
    }
    cells[k] = make_float2((float)c0, (float)c1);
  }
  __syncthreads();
  const float wscale = g_wscale;

  // ---- staging: per warp two tiles of WT = VF_MAP_EPT * 32 events, each
  // [x: WT*D floats][ind: WT*D ints][w: WT floats]
  const bool want_ind = ind_out != nullptr;
  unsigned char* stage0 = smem + ((NB * 8 + 15) & ~15);
  const bool aligned = ((reinterpret_cast<size_t>(x_out) | reinterpret_cast<size_t>(w_out) |
                         reinterpret_cast<size_t>(ind_out)) & 15) == 0;
  const long long n = a.n_events;
  // a warp hands its own tiles to the copy engine: no block-wide barrier
  const int lane = tid & 31, warp = tid >> 5;
  constexpr int WT = VF_MAP_EPT * 32;
  constexpr u32 XBW = WT * D * 4, WBW = WT * 4;
  const u32 wstage = XBW * (want_ind ? 2u : 1u) + WBW;
  unsigned char* wbase = stage0 + (size_t)warp * 2 * wstage;
  const long long n_wt = (n + WT - 1) / WT;
  int it = 0;
  for (long long t = (long long)blockIdx.x * (THREADS / 32) + warp; t < n_wt;
       t += (long long)gridDim.x * (THREADS / 32), ++it) {
    const long long e0 = t * WT;
    const bool full = aligned && e0 + WT <= n;  // warp-uniform
    unsigned char* st = wbase + (it & 1) * wstage;
    u32* xs = reinterpret_cast<u32*>(st);
    u32* is = reinterpret_cast<u32*>(st + XBW);
    float* wsm = reinterpret_cast<float*>(st + XBW * (want_ind ? 2 : 1));
    if (full) {
      // the stage's previous tile (two tiles back) must have been read out
      if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
      __syncwarp();
    }
#pragma unroll
    for (int k = 0; k < VF_MAP_EPT; ++k) {
      const int r = k * 32 + lane;  // row in the warp's tile
      const long long e = e0 + r;
      if (e < n) {
        const u64 ev = (u64)(a.ev_offset + e);
        float wf = 1.0f;
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
              const u64 pp = (u64)(~wq[j]) * 50ull + 25ull;
              const int i = (int)(pp >> 32);
              const float m = __uint_as_float(((u32)pp >> 9) | 0x3F800000u);
              const float2 c = cells[d * VF_BINS + i];
              xr[d] = __float_as_uint(fmaf(c.y, m, c.x));
              wf = (d == 0) ? c.y : wf * c.y;
              br[d] = (u32)i;
            }
          }
        }
        const float w = wf * wscale;
        if (full) {
          stage_row<D>(xs + r * D, xr);
          if (want_ind) stage_row<D>(is + r * D, br);
          wsm[r] = w;
        } else {
          if (x_out)
#pragma unroll
            for (int d = 0; d < D; ++d) x_out[e * D + d] = __uint_as_float(xr[d]);
          if (want_ind)
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
        if (want_ind) bulk_store(ind_out + e0 * D, smem_u32(is), XBW);
        if (w_out) bulk_store(w_out + e0, smem_u32(wsm), WBW);
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      }
    }
  }
  if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

}  // namespace vf
