// gt_serve.cu -- device-side inputs of served requests, and plain device
// buffers from a context's pool.
//
// A served request is described by its seed: its per-cell coefficient is
// the seeded lognormal field exp(sigma z_c), z_c the Box-Muller normal of two
// counter-based uniforms.  Generating it on the device keeps the request's
// host work to one call (no host arrays, no upload): under a request stream
// the host side of a server is shared by all its slots, so every host
// microsecond per request counts.
#include <cmath>

#include "gt_internal.cuh"

namespace gt {

// splitmix64 (Steele, Lea, Flood 2014): the finaliser of a Weyl sequence,
// used as a keyed hash: u(seed, key) = (splitmix64(seed ^ key) >> 11) 2^-53
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  uint64_t z = x;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double keyed_uniform(uint64_t seed, uint64_t key) {
  return (double)(splitmix64(seed ^ key) >> 11) * 0x1.0p-53;
}

// out[c] = exp(sigma sqrt(-2 log(1 - u(s, 2c))) cos(2 pi u(s, 2c + 1)))
__global__ void k_lognormal_cells(int64_t n, double sigma, uint64_t s, double* __restrict__ out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const double u1 = keyed_uniform(s, 2 * (uint64_t)c), u2 = keyed_uniform(s, 2 * (uint64_t)c + 1);
    const double z = sqrt(-2.0 * log(1.0 - u1)) * cos(6.283185307179586 * u2);
    out[c] = exp(sigma * z);
  }
}

}  // namespace gt

using namespace gt;

extern "C" {

int gt_device_alloc(gt_ctx* ctx, int64_t bytes, void** out) {
  if (!ctx || !out || bytes < 0) return GT_ERR_INVALID;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  unsigned char* p = nullptr;
  GT_TRY(dalloc(ctx, &p, bytes));
  *out = p;
  return GT_OK;
}

int gt_device_free(gt_ctx* ctx, void* p) {
  if (!ctx) return GT_ERR_INVALID;
  pool_free(ctx, p);
  return GT_OK;
}

int gt_device_copy(gt_ctx* ctx, void* dst, const void* src, int64_t bytes) {
  if (!ctx || (bytes > 0 && (!dst || !src)) || bytes < 0) return GT_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (bytes == 0) return GT_OK;
  GT_CUDA(ctx, cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDefault, ctx->stream));
  GT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GT_OK;
}

int gt_lognormal_cells(gt_ctx* ctx, int64_t ncells, double sigma, uint64_t seed, double* out) {
  if (!ctx || ncells < 0 || (ncells > 0 && !out)) return GT_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (ncells == 0) return GT_OK;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, out) != cudaSuccess || at.type != cudaMemoryTypeDevice ||
      at.device != ctx->device) {
    cudaGetLastError();
    return set_error(ctx, GT_ERR_INVALID, "gt_lognormal_cells: out must be device memory of the context's device");
  }
  const uint64_t s = seed ^ 0xC0EFF1C1E47ull;
  k_lognormal_cells<<<GT_KC(ctx, grid_for(ncells, 256)), 256, 0, ctx->stream>>>(ncells, sigma, s, out);
  GT_LAUNCH(ctx, "k_lognormal_cells");
  return GT_OK;
}

}  // extern "C"
