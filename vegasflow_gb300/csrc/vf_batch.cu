// Batched-VEGAS entry points (vf_batch_*): many integrals per launch.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>

#include "vegasflow_gb300.h"
#include "vf_batch.cuh"
#include "vf_internal.h"

static_assert(sizeof(vf_batch_item) == sizeof(vf::BatchItem), "vf_batch_item layout");

namespace {

int err(int code, const char* msg) { return vf::set_error(code, msg); }

int launched(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return err(VF_ERR_LAUNCH, buf);
  }
  return VF_OK;
}

// The device address of `p`: `p` itself for device memory, the mapped address
// for pinned host memory (the same pointer under unified addressing).
bool device_address(double* p, double** out) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess || at.devicePointer == nullptr ||
      (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeHost && at.type != cudaMemoryTypeManaged)) {
    cudaGetLastError();  // clear the lookup's error
    return false;
  }
  *out = static_cast<double*>(at.devicePointer);
  return true;
}

// The sampler of a dimension class (n_dim <= 8, or any).
const void* sample_kernel_for(int max_dim) {
  return max_dim <= 8 ? (const void*)vf::vf_batch_sample_kernel<8> : (const void*)vf::vf_batch_sample_kernel<16>;
}

// Raise a sampler's dynamic shared-memory limit once per size (a no-op
// afterwards, so launches inside a stream capture make no attribute calls).
std::atomic<int> g_smem_set[2] = {{0}, {0}};
cudaError_t set_smem(int max_dim, int smem) {
  std::atomic<int>& done = g_smem_set[max_dim <= 8 ? 0 : 1];
  if (smem <= done.load()) return cudaSuccess;
  const cudaError_t e =
      cudaFuncSetAttribute(sample_kernel_for(max_dim), cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) done.store(smem);
  return e;
}

}  // namespace

extern "C" {

int vf_batch_blocks(int max_dim, int* blocks, int* smem_bytes) {
  if (!blocks || max_dim < 1 || max_dim > VF_MAX_DIM) return err(VF_ERR_ARG, "vf_batch_blocks: max_dim");
  const int smem = vf::batch_smem_bytes(max_dim);
  cudaError_t e = set_smem(max_dim, smem);
  if (e != cudaSuccess) return err(VF_ERR_CUDA, cudaGetErrorString(e));
  // load the batch kernels now, so that a later stream capture launches only
  if (vf::preload_batch_kernels() != cudaSuccess)
    return err(VF_ERR_CUDA, "vf_batch_blocks: loading the batch kernels failed");
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sample_kernel_for(max_dim), VF_THREADS, smem);
  if (e != cudaSuccess) return err(VF_ERR_CUDA, cudaGetErrorString(e));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  *blocks = (per_sm > 0 ? per_sm : 1) * sms;
  if (smem_bytes) *smem_bytes = smem;
  return VF_OK;
}

}  // extern "C"

namespace {

// The sampler arguments shared by vf_batch_sample and vf_batch_sample_jit.
int batch_args(vf::BatchArgs& a, const vf_batch_item* items, const int* tile_item, const long long* tile_start,
               const int* tile_count, const long long* tile_row, int n_tiles, int max_dim, int* queue,
               const unsigned int* calls, const double* grids, const double* params, double* partials,
               unsigned long long seed, int* flags, int blocks) {
  if (!items || !tile_item || !tile_start || !tile_count || !tile_row || !queue || !calls || !grids ||
      !params || !partials || n_tiles < 0 || blocks < 1)
    return err(VF_ERR_ARG, "vf_batch_sample: NULL buffer or bad sizes");
  if (max_dim < 1 || max_dim > VF_MAX_DIM) return err(VF_ERR_UNSUPPORTED, "vf_batch_sample: max_dim must be 1..16");
  a.items = reinterpret_cast<const vf::BatchItem*>(items);
  a.tile_item = tile_item;
  a.tile_start = tile_start;
  a.tile_count = tile_count;
  a.tile_row = tile_row;
  a.queue = queue;
  a.calls = calls;
  a.grids = grids;
  a.params = params;
  a.partials = partials;
  a.flags = flags;
  a.n_tiles = n_tiles;
  a.max_dim = max_dim;
  unsigned int k0 = (unsigned int)seed, k1 = (unsigned int)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    a.rk.k0[r] = k0;
    a.rk.k1[r] = k1;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return VF_OK;
}

}  // namespace

extern "C" {

int vf_batch_sample(const vf_batch_item* items, const int* tile_item, const long long* tile_start,
                    const int* tile_count, const long long* tile_row, int n_tiles, int max_dim, int* queue,
                    const unsigned int* calls, const double* grids, const double* params, double* partials,
                    unsigned long long seed, int* flags, int blocks, void* stream) {
  vf::BatchArgs a;
  const int rc = batch_args(a, items, tile_item, tile_start, tile_count, tile_row, n_tiles, max_dim, queue, calls,
                            grids, params, partials, seed, flags, blocks);
  if (rc != VF_OK) return rc;
  const int smem = vf::batch_smem_bytes(max_dim);
  cudaError_t e = set_smem(max_dim, smem);
  if (e != cudaSuccess) return err(VF_ERR_CUDA, cudaGetErrorString(e));
  void* args[] = {&a};
  e = cudaLaunchKernel(sample_kernel_for(max_dim), dim3(blocks), dim3(VF_THREADS), args, smem, (cudaStream_t)stream);
  if (e != cudaSuccess) return err(VF_ERR_LAUNCH, cudaGetErrorString(e));
  return launched("vf_batch_sample");
}

int vf_batch_sample_jit(int integrand_id, const vf_batch_item* items, const int* tile_item,
                        const long long* tile_start, const int* tile_count, const long long* tile_row, int n_tiles,
                        int max_dim, int* queue, const unsigned int* calls, const double* grids, const double* params,
                        double* partials, unsigned long long seed, int* flags, int blocks, void* stream) {
  vf::BatchArgs a;
  const int rc = batch_args(a, items, tile_item, tile_start, tile_count, tile_row, n_tiles, max_dim, queue, calls,
                            grids, params, partials, seed, flags, blocks);
  if (rc != VF_OK) return rc;
  const int rl = vf::jit_launch_batch(integrand_id, max_dim, &a, blocks, vf::batch_smem_bytes(max_dim), stream);
  if (rl != VF_OK) return rl;
  return launched("vf_batch_sample_jit");
}

int vf_batch_iteration_end(const vf_batch_item* items, const int* blk_item, const int* blk_role, int n_blocks,
                           const long long* tile_row, const double* partials, double* grids, double* history,
                           double* avg, int hist_cap, int* iters, unsigned int* calls, int* queue, int* flags,
                           double* status, void* stream) {
  if (!items || !blk_item || !blk_role || !tile_row || !partials || !grids || !history || !avg || !iters ||
      !calls || !queue ||
      n_blocks < 1 || hist_cap < 1)
    return err(VF_ERR_ARG, "vf_batch_iteration_end: NULL buffer or bad sizes");
  double* status_dev = nullptr;
  if (status && !device_address(status, &status_dev))
    return err(VF_ERR_ARG, "vf_batch_iteration_end: status is neither device memory nor host memory the device "
                           "can address");
  vf::BatchEndArgs a;
  a.items = reinterpret_cast<const vf::BatchItem*>(items);
  a.blk_item = blk_item;
  a.blk_role = blk_role;
  a.tile_row = tile_row;
  a.partials = partials;
  a.grids = grids;
  a.history = history;
  a.avg = avg;
  a.iters = iters;
  a.calls = calls;
  a.queue = queue;
  a.flags = flags;
  a.status = status_dev;
  a.alpha = 1.5;
  a.hist_cap = hist_cap;
  vf::vf_batch_end_kernel<<<n_blocks, VF_BATCH_END_THREADS, 0, (cudaStream_t)stream>>>(a);
  return launched("vf_batch_iteration_end");
}

}  // extern "C"

namespace vf {
cudaError_t preload_batch_kernels() {
  cudaFuncAttributes attr;
  cudaError_t e = cudaFuncGetAttributes(&attr, vf_batch_sample_kernel<8>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&attr, vf_batch_sample_kernel<16>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&attr, vf_batch_end_kernel);
  return e;
}
}  // namespace vf
