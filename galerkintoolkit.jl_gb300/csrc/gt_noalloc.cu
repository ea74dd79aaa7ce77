// gt_noalloc.cu -- matrix refill that allocates no device memory.
//
// gt_update_matrix_noalloc recomputes the values of an assembled matrix on
// its existing sparsity, like gt_update_matrix, but takes its scratch (the
// reference-cell tabulation and the element matrices that the row-owner
// scatter reads) from one fixed, file-scope device array instead of the
// context's buffer pool.  It is meant for callers that cannot let the
// library allocate:
//   * processes whose device memory is budgeted up front -- a serving loop
//     whose admission control has already accounted every byte, or a host
//     runtime whose own memory pool owns the device (a Julia/CUDA.jl or
//     PyTorch process), where a cudaMalloc behind its back breaks the budget;
//   * latency-critical refill loops (Newton or time-stepping updates of the
//     same matrix), where a cudaMalloc/cudaFree can synchronise the device.
// The caller provides every input and output in device memory: the matrix
// (already assembled, so its sparsity and value arrays exist) and the
// per-cell coefficient (device pointer or NULL).
//
// Limits and sharing:
//   * the array holds kNoAllocScratchBytes (128 MiB); a refill needing more
//     (tabulation + ncells * nloc^2 values) is rejected with GT_ERR_INVALID;
//   * every GPU that loads the library holds the array until process exit;
//   * all calls share the one array and it keeps the last call's contents;
//     nothing in it needs to start at zero because each call writes every
//     element it reads before reading it; calls that overlap on the GPU
//     (two streams or two contexts at once) race on the array -- serialise
//     them;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress with that device current, the caller's current
//     device restored afterwards);
//   * every call waits for the context's stream before it returns (it reads
//     the kernels' error word).
#include <mutex>

#include "gt_internal.cuh"

namespace gt {

constexpr size_t kNoAllocScratchBytes = size_t(128) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_refill_scratch[kNoAllocScratchBytes];

static std::mutex g_setup_mutex;
static void* g_scratch_addr[kMaxDevices] = {nullptr};

// device address of the scratch array on the current device (set-up once)
static int scratch_address(Ctx* ctx, void** out) {
  if (ctx->device < 0 || ctx->device >= kMaxDevices) return set_error(ctx, GT_ERR_INVALID, "device id out of range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[ctx->device]) {
    int prev = 0;
    GT_CUDA(ctx, cudaGetDevice(&prev));
    GT_CUDA(ctx, cudaSetDevice(ctx->device));
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_refill_scratch);
    cudaSetDevice(prev);
    if (e != cudaSuccess || !p) return check_cuda(ctx, e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress");
    g_scratch_addr[ctx->device] = p;
  }
  *out = g_scratch_addr[ctx->device];
  return GT_OK;
}

}  // namespace gt

using namespace gt;

extern "C" {

int gt_update_matrix_noalloc(gt_matrix* A, int form, const double* cell_coef, double nu) {
  if (!A) return GT_ERR_INVALID;
  Ctx* ctx = A->ctx;
  const Space* sp = A->space;
  if (!A->colind || (!A->val64 && !A->val32))
    return set_error(ctx, GT_ERR_INVALID, "gt_update_matrix_noalloc needs an assembled matrix");
  if (cell_coef) {
    cudaPointerAttributes at{};
    cudaError_t e = cudaPointerGetAttributes(&at, cell_coef);
    if (e != cudaSuccess || (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
      cudaGetLastError();
      return set_error(ctx, GT_ERR_INVALID, "gt_update_matrix_noalloc: cell_coef must be device memory (or NULL)");
    }
    if (at.type == cudaMemoryTypeDevice && at.device != ctx->device)
      return set_error(ctx, GT_ERR_INVALID, "gt_update_matrix_noalloc: cell_coef is memory of another device");
  }
  int kprec = A->precision == GT_FP32 ? GT_FP32 : GT_FP64;
  size_t esz = kprec == GT_FP32 ? sizeof(float) : sizeof(double);
  size_t tab_bytes = ((size_t)tabulation_doubles(sp) * sizeof(double) + 255) & ~size_t(255);
  size_t ke_bytes = (size_t)sp->mesh->ncells * ke_per_cell(sp) * esz;
  if (tab_bytes + ke_bytes > kNoAllocScratchBytes)
    return set_error(ctx, GT_ERR_INVALID,
                     "gt_update_matrix_noalloc: needs " + std::to_string(tab_bytes + ke_bytes) +
                         " bytes of scratch; the static limit is " + std::to_string(kNoAllocScratchBytes) +
                         " bytes (use gt_update_matrix)");
  void* base = nullptr;
  GT_TRY(scratch_address(ctx, &base));
  GT_CUDA(ctx, cudaSetDevice(ctx->device));
  double* tab = (double*)base;
  void* Ke = (unsigned char*)base + tab_bytes;
  GT_TRY(compute_elements_with_tab(sp, form, cell_coef, nu, A->precision, tab, Ke));
  GT_TRY(scatter_matrix(A, Ke, kprec, A->precision));
  uint32_t bits = 0;
  GT_TRY(take_device_error(ctx, &bits));  // synchronises the stream
  if (bits & DEV_ERR_DEGENERATE) return set_error(ctx, GT_ERR_INVALID, "gt_update_matrix_noalloc: degenerate cell");
  if (bits) return set_error(ctx, GT_ERR_INVALID, "gt_update_matrix_noalloc: device-side check failed");
  return GT_OK;
}

}  // extern "C"
