// Host-side internal declarations shared by the translation units of
// libvegasgb.so (not part of the public C-ABI).
#pragma once
#include <cuda_runtime.h>

namespace vf {

// Kernel pointers of the ahead-of-time sampler instantiations
// (dmax in {4, 8, 16}; integrand a VF_INT_* id), or nullptr.
const void* sample_kernel_f64(int dmax, int integrand);
const void* sample_kernel_f32(int dmax, int integrand);

// The fp32 VEGAS Philox sampler specialised on the exact dimension count and
// the block size (1024 or 512 threads), one function per instantiation unit.
const void* vegas_f32_kernel_t1024_1_4(int n_dim, int integrand);
const void* vegas_f32_kernel_t1024_5_8(int n_dim, int integrand);
const void* vegas_f32_kernel_t1024_9_12(int n_dim, int integrand);
const void* vegas_f32_kernel_t1024_13_16(int n_dim, int integrand);
const void* vegas_f32_kernel_t512_1_8(int n_dim, int integrand);
const void* vegas_f32_kernel_t512_9_16(int n_dim, int integrand);
inline const void* vegas_f32_kernel(int n_dim, int integrand, int threads) {
  if (threads == 512) return n_dim <= 8 ? vegas_f32_kernel_t512_1_8(n_dim, integrand)
                                        : vegas_f32_kernel_t512_9_16(n_dim, integrand);
  if (threads != 1024) return nullptr;
  if (n_dim <= 4) return vegas_f32_kernel_t1024_1_4(n_dim, integrand);
  if (n_dim <= 8) return vegas_f32_kernel_t1024_5_8(n_dim, integrand);
  if (n_dim <= 12) return vegas_f32_kernel_t1024_9_12(n_dim, integrand);
  return vegas_f32_kernel_t1024_13_16(n_dim, integrand);
}

// The fp32 VEGAS sampler for injected float64 uniforms (VF_INJ_THREADS per block);
// `tap`: its parity instantiation (VF_INT_SYMGAUSS and VF_INT_PROD only).
const void* vegas_f32_inj_kernel_d1_8(int n_dim, int integrand, bool tap);
const void* vegas_f32_inj_kernel_d9_16(int n_dim, int integrand, bool tap);
inline const void* vegas_f32_inj_kernel(int n_dim, int integrand, bool tap) {
  return n_dim <= 8 ? vegas_f32_inj_kernel_d1_8(n_dim, integrand, tap)
                    : vegas_f32_inj_kernel_d9_16(n_dim, integrand, tap);
}

// The parity instantiation of the fp32 VEGAS Philox sampler (1024 threads; writes each
// event's bin indices): VF_INT_SYMGAUSS and VF_INT_PROD, dimensions 1..16.
const void* vegas_f32_tap_kernel(int n_dim, int integrand);

// The fp32 VEGAS+ sampler for built-in integrands, specialised on the
// dimension count (Philox uniforms; 256 threads per block).
const void* plus_f32_kernel(int n_dim, int integrand);
// Its parity instantiation (writes bin indices and float32 points):
// VF_INT_SYMGAUSS and VF_INT_BREIT_WIGNER, dimensions 1..16.
const void* plus_f32_tap_kernel(int n_dim, int integrand);

// The fp32 VEGAS map kernel without an integrand (x, w and, with `ind`, bin
// indices to HBM), specialised on the dimension count; VF_MAP_THREADS per block.
const void* vegas_f32_map_kernel(int n_dim, bool ind);

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
