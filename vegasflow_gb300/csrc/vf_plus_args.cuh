// The argument block of the VEGAS+ samplers (float64 and fp32 kernels).
#pragma once
#include "vf_sample.cuh"

namespace vf {

struct PlusArgs {
  const double* grid;        // [D][51]
  const int* n_ev;           // [H]
  const long long* ev_start; // [H + 1]
  const double* xmin;        // nullable [D]
  const double* xdelta;      // nullable [D]
  const double* u_inj;       // nullable [n_events][D] (post-affine uniforms, event order)
  const double* params;
  double* ress;              // [H]: sum of w f per hypercube (nullable when sampling only)
  double* ress2;             // [H]: sum of (w f)^2
  double* partials;          // [rows][2 + 50 D]: block sums and histogram
  int* ind_out;              // nullable taps, indexed by event
  void* x_out;
  void* w_out;
  int* flags;
  double xjac;               // 1 / n_hypercubes (vflowplus.py:139, :144-146)
  double xdeltajac;
  int n_dim;
  int n_strat;
  int n_hcubes;
  int train;
  RoundKeys rk;
  unsigned int ctr2[8];
  unsigned int ctr3;
  const unsigned int* call_dev;  // nullable: the Philox call counter in device memory (graph replays)
};

// Philox counter words of this iteration: word 2 without the block index q
// (word 2 = base | q) and word 3, from the device call counter when there is
// one, else as the host computed them.
__device__ __forceinline__ void plus_call_words(const PlusArgs& a, unsigned int& c2base, unsigned int& c3) {
  if (a.call_dev) {
    const unsigned int call = *a.call_dev;
    c2base = call << 4;
    c3 = call >> 28;
  } else {
    c2base = a.ctr2[0];
    c3 = a.ctr3;
  }
}

__host__ __device__ inline int plus_smem_bytes(int real_size, int D, int train) {
  return D * VF_EDGES * 8 + (train ? D * VF_BINS * real_size : 0) + 2 * VF_MAX_DIM * 8;
}

}  // namespace vf
