// Host-side internal declarations shared by the translation units of
// libvegasgb.so (not part of the public C-ABI).
#pragma once
#include <cuda_runtime.h>

namespace vf {

// Kernel pointers of the ahead-of-time sampler instantiations
// (dmax in {4, 8, 16}; integrand a VF_INT_* id), or nullptr.
const void* sample_kernel_f64(int dmax, int integrand);
const void* sample_kernel_f32(int dmax, int integrand);

// The fp32 VEGAS sampler specialised on the exact dimension count (1..8 in
// part a, 9..16 in part b) and the block size (128 or 256 threads).
const void* vegas_f32_kernel_a256(int n_dim, int integrand);
const void* vegas_f32_kernel_b256(int n_dim, int integrand);
const void* vegas_f32_kernel_a128(int n_dim, int integrand);
const void* vegas_f32_kernel_b128(int n_dim, int integrand);
inline const void* vegas_f32_kernel(int n_dim, int integrand, int threads = 256) {
  if (threads == 128)
    return n_dim <= 8 ? vegas_f32_kernel_a128(n_dim, integrand) : vegas_f32_kernel_b128(n_dim, integrand);
  return n_dim <= 8 ? vegas_f32_kernel_a256(n_dim, integrand) : vegas_f32_kernel_b256(n_dim, integrand);
}

// The parity instantiation of the fp32 VEGAS sampler (256 threads; writes each
// event's bin indices): VF_INT_SYMGAUSS and VF_INT_PROD, dimensions 1..16.
const void* vegas_f32_tap_kernel(int n_dim, int integrand);

// The fp32 VEGAS+ sampler for built-in integrands, specialised on the
// dimension count (Philox uniforms; 256 threads per block).
const void* plus_f32_kernel(int n_dim, int integrand);
// Its parity instantiation (writes bin indices and float32 points):
// VF_INT_SYMGAUSS and VF_INT_BREIT_WIGNER, dimensions 1..16.
const void* plus_f32_tap_kernel(int n_dim, int integrand);

// The fp32 VEGAS map kernel without an integrand (x, w, bin indices to HBM),
// specialised on the dimension count; 256 threads per block.
const void* vegas_f32_map_kernel(int n_dim);

// Launches the NVRTC-compiled sampler of a JIT integrand with `args` (a
// SampleArgs); reports whether it is the fp32 VEGAS kernel and settles the
// histogram layout it uses.
int jit_launch(int integrand_id, int alg, int precision, int n_dim, void* args, int rows, int train,
               void* stream, int* fast_out, int* hist_copies_inout);

// Load (cudaFuncGetAttributes) every kernel of a translation unit on the
// current device; return the first CUDA error, or cudaSuccess.
cudaError_t preload_plus_kernels();
cudaError_t preload_batch_kernels();
cudaError_t preload_probe_kernels();

// Launches the NVRTC-compiled VEGAS+ sampler of a JIT integrand with `args` (a
// PlusArgs): the float32 one when `use_fast` and it exists, else the generic one.
int jit_launch_plus(int integrand_id, int precision, int n_dim, void* args, int rows, int train, bool use_fast,
                    void* stream);

// Launches the NVRTC-compiled batched sampler of a JIT integrand with `args` (a
// BatchArgs) on `blocks` blocks with `smem` bytes of dynamic shared memory; the
// integrand must have been compiled for integrals of at least `max_dim` dimensions.
int jit_launch_batch(int integrand_id, int max_dim, void* args, int blocks, int smem, void* stream);

// Records an error message for vf_last_error_string(); returns `code`.
int set_error(int code, const char* message);

inline int dim_bucket(int n_dim) { return n_dim <= 4 ? 4 : (n_dim <= 8 ? 8 : 16); }

}  // namespace vf
