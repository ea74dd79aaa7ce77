// gt_context.cu -- context, device buffer pool, error plumbing, scans.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "gt_internal.cuh"

namespace gt {

int set_error(Ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int check_cuda(Ctx* ctx, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return set_error(ctx, GT_ERR_OOM, m);
  return set_error(ctx, GT_ERR_CUDA, m);
}

// Blocks are pooled by exact size class (rounded up to 2 MiB above 1 MiB,
// to 256 B below) so that repeated assemblies of the same problem reuse
// their buffers without cudaMalloc/cudaFree, which synchronise the device.
static size_t size_class(size_t b) {
  if (b <= (1u << 20)) return (b + 255) & ~size_t(255);
  size_t g = size_t(2) << 20;
  return (b + g - 1) / g * g;
}

void* pool_alloc(Ctx* ctx, size_t bytes) {
  // every block has at least 16 bytes past its end: bulk (TMA) copies of a
  // segment round its end up to a 16-byte boundary
  size_t sc = size_class(bytes + 16);
  auto it = ctx->pool.lower_bound(sc);
  if (it != ctx->pool.end() && it->first <= sc + sc / 4) {
    void* p = it->second;
    size_t s = it->first;
    ctx->pool.erase(it);
    ctx->pooled_bytes -= (int64_t)s;
    ctx->live[p] = s;
    ctx->live_bytes += (int64_t)s;
    return p;
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, sc);
  if (e != cudaSuccess) {
    cudaGetLastError();
    pool_trim(ctx);
    e = cudaMalloc(&p, sc);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
  }
  ctx->live[p] = sc;
  ctx->live_bytes += (int64_t)sc;
  return p;
}

void pool_free(Ctx* ctx, void* p) {
  auto it = ctx->live.find(p);
  if (it == ctx->live.end()) return;
  size_t s = it->second;
  ctx->live.erase(it);
  ctx->live_bytes -= (int64_t)s;
  ctx->pool.emplace(s, p);
  ctx->pooled_bytes += (int64_t)s;
}

void pool_trim(Ctx* ctx) {
  if (ctx->pool.empty()) return;
  cudaStreamSynchronize(ctx->stream);
  if (ctx->aux) cudaStreamSynchronize(ctx->aux);
  for (auto& kv : ctx->pool) cudaFree(kv.second);
  ctx->pool.clear();
  ctx->pooled_bytes = 0;
}

cudaEvent_t event_get(Ctx* ctx) {
  if (!ctx->free_events.empty()) {
    cudaEvent_t e = ctx->free_events.back();
    ctx->free_events.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return e;
}

void event_put(Ctx* ctx, cudaEvent_t e) {
  if (e) ctx->free_events.push_back(e);
}

int side_copy_in(Ctx* ctx, void* dst, const void* src, size_t bytes, cudaEvent_t* done) {
  *done = nullptr;
  cudaEvent_t after = event_get(ctx), ev = event_get(ctx);
  if (!after || !ev) return set_error(ctx, GT_ERR_CUDA, "cudaEventCreate failed");
  GT_CUDA(ctx, cudaEventRecord(after, ctx->stream));
  GT_CUDA(ctx, cudaStreamWaitEvent(ctx->side, after, 0));
  GT_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->side));
  GT_CUDA(ctx, cudaEventRecord(ev, ctx->side));
  event_put(ctx, after);  // the wait above captured its state: reusable
  *done = ev;
  return GT_OK;
}

void mesh_wait_coords(Mesh* m) {
  if (m->coords_pending && m->coords_ev) {
    cudaStreamWaitEvent(m->ctx->stream, m->coords_ev, 0);
    m->coords_pending = false;
  }
}

void mesh_wait_coords_on(Mesh* m, cudaStream_t s) {
  if (m->coords_pending && m->coords_ev) cudaStreamWaitEvent(s, m->coords_ev, 0);
}

void mark(Ctx* ctx, const char* name) {
  if (!ctx->prof) return;
  cudaEvent_t e;
  if (!ctx->spare_events.empty()) {
    e = ctx->spare_events.back();
    ctx->spare_events.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  cudaEventRecord(e, ctx->stream);
  ctx->marks.emplace_back(name, e);
}

int take_device_error(Ctx* ctx, uint32_t* bits) {
  GT_CUDA(ctx, cudaMemcpyAsync(ctx->h_err, ctx->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  GT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const uint32_t dev = *ctx->h_err;
  *bits = dev | ctx->held_err;
  ctx->held_err = 0;
  if (dev) GT_CUDA(ctx, cudaMemsetAsync(ctx->d_err, 0, sizeof(uint32_t), ctx->stream));
  return GT_OK;
}

// ---------------------------------------------------------------------------
// exclusive scan: per-block sums, recursive scan of the sums, then a block
// scan that adds the block offset.  2048 items per block of 256 threads.
// ---------------------------------------------------------------------------
constexpr int SCAN_T = 256, SCAN_V = 8, SCAN_B = SCAN_T * SCAN_V;

template <class Tin, class Tout>
__global__ void k_block_sums(const Tin* __restrict__ in, Tout* __restrict__ sums, int64_t n) {
  __shared__ Tout red[SCAN_T / 32];
  int64_t base = (int64_t)blockIdx.x * SCAN_B;
  Tout s = 0;
#pragma unroll
  for (int v = 0; v < SCAN_V; v++) {
    int64_t i = base + (int64_t)v * SCAN_T + threadIdx.x;
    if (i < n) s += (Tout)in[i];
  }
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    Tout t = 0;
    for (int w = 0; w < SCAN_T / 32; w++) t += red[w];
    sums[blockIdx.x] = t;
  }
}

template <class Tin, class Tout>
__global__ void k_block_scan(const Tin* __restrict__ in, Tout* __restrict__ out, const Tout* __restrict__ offs,
                             int64_t n) {
  __shared__ Tout warp_tot[SCAN_T / 32];
  int64_t base = (int64_t)blockIdx.x * SCAN_B + (int64_t)threadIdx.x * SCAN_V;
  Tout v[SCAN_V];
  Tout t = 0;
#pragma unroll
  for (int k = 0; k < SCAN_V; k++) {
    int64_t i = base + k;
    v[k] = i < n ? (Tout)in[i] : (Tout)0;
    t += v[k];
  }
  // inclusive warp scan of thread totals
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  Tout x = t;
  for (int o = 1; o < 32; o <<= 1) {
    Tout y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  Tout wo = 0;
  for (int k = 0; k < w; k++) wo += warp_tot[k];
  Tout run = (offs ? offs[blockIdx.x] : (Tout)0) + wo + x - t;
#pragma unroll
  for (int k = 0; k < SCAN_V; k++) {
    int64_t i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == SCAN_T - 1) out[n] = run;
}

template <class Tin, class Tout>
static int scan_impl(Ctx* ctx, const Tin* in, Tout* out, int64_t n) {
  if (n <= 0) {
    GT_CUDA(ctx, cudaMemsetAsync(out, 0, sizeof(Tout), ctx->stream));
    return GT_OK;
  }
  int64_t nb = (n + SCAN_B - 1) / SCAN_B;
  if (nb == 1) {
    k_block_scan<Tin, Tout><<<GT_KC(ctx, 1), SCAN_T, 0, ctx->stream>>>(in, out, nullptr, n);
    GT_LAUNCH(ctx, "k_block_scan");
    return GT_OK;
  }
  Tout* sums = nullptr;
  Tout* soff = nullptr;
  GT_TRY(dalloc(ctx, &sums, nb));
  GT_TRY(dalloc(ctx, &soff, nb + 1));
  k_block_sums<Tin, Tout><<<GT_KC(ctx, (unsigned)nb), SCAN_T, 0, ctx->stream>>>(in, sums, n);
  GT_LAUNCH(ctx, "k_block_sums");
  int s = scan_impl<Tout, Tout>(ctx, sums, soff, nb);
  if (s == GT_OK) {
    k_block_scan<Tin, Tout><<<GT_KC(ctx, (unsigned)nb), SCAN_T, 0, ctx->stream>>>(in, out, soff, n);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) s = check_cuda(ctx, e, "k_block_scan");
  }
  dfree(ctx, sums);
  dfree(ctx, soff);
  return s;
}

int exclusive_scan_i64(Ctx* ctx, const int32_t* in, int64_t* out, int64_t n) {
  return scan_impl<int32_t, int64_t>(ctx, in, out, n);
}
int exclusive_scan_i32(Ctx* ctx, const int32_t* in, int32_t* out, int64_t n) {
  return scan_impl<int32_t, int32_t>(ctx, in, out, n);
}

// FMA throughput probe: 8 independent FMA chains per thread, a full wave of
// CTAs on every SM; used to state the FP32/FP64 pipe roofline of the
// integration kernels on the running device.
template <class T>
__global__ void k_fma_rate(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <class T>
static int fma_rate(Ctx* ctx, int iters, double* tflops) {
  int blocks = ctx->num_sms * 8, threads = 256;
  T* out = nullptr;
  GT_TRY(dalloc(ctx, &out, (int64_t)blocks * threads));
  cudaEvent_t e0, e1;
  GT_CUDA(ctx, cudaEventCreate(&e0));
  GT_CUDA(ctx, cudaEventCreate(&e1));
  k_fma_rate<T><<<GT_KC(ctx, blocks), threads, 0, ctx->stream>>>(out, iters / 4, (T)0.999, (T)0.001);
  cudaEventRecord(e0, ctx->stream);
  k_fma_rate<T><<<GT_KC(ctx, blocks), threads, 0, ctx->stream>>>(out, iters, (T)0.999, (T)0.001);
  cudaEventRecord(e1, ctx->stream);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dfree(ctx, out);
  if (e != cudaSuccess) return check_cuda(ctx, e, "k_fma_rate");
  *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
  return GT_OK;
}

}  // namespace gt

using namespace gt;

extern "C" {

int gt_ctx_create(int device, gt_ctx** out) {
  if (!out) return GT_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return GT_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return GT_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return GT_ERR_CUDA;
  gt_ctx* c = new gt_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  // the auxiliary compute stream takes the lowest priority and the main
  // stream the highest: pending blocks of the main stream's kernels (the
  // sparsity kernels, whose result the host downloads first) are dispatched
  // before those of the element kernels beside them
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  if (cudaStreamCreateWithPriority(&c->own_stream, cudaStreamNonBlocking, prio_greatest) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->aux, cudaStreamNonBlocking, prio_least) != cudaSuccess ||
      cudaMalloc(&c->d_err, sizeof(uint32_t)) != cudaSuccess ||
      cudaMallocHost(&c->h_err, sizeof(uint32_t)) != cudaSuccess ||
      cudaMallocHost(&c->h_scratch, 64 * sizeof(int64_t)) != cudaSuccess ||
      cudaMallocHost(&c->h_dscratch, 64 * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->aux) cudaStreamDestroy(c->aux);
    if (c->d_err) cudaFree(c->d_err);
    if (c->h_err) cudaFreeHost(c->h_err);
    if (c->h_scratch) cudaFreeHost(c->h_scratch);
    delete c;
    return GT_ERR_CUDA;
  }
  c->stream = c->own_stream;
  const char* pcg = getenv("GTGPU_PCG");
  c->pcg_path = !pcg ? 0 : strcmp(pcg, "launches") == 0 ? 1 : strcmp(pcg, "persistent") == 0 ? 2 : 0;
  const char* ov = getenv("GTGPU_OVERLAP");
  c->overlap = !(ov && strcmp(ov, "0") == 0);
  const char* pt = getenv("GTGPU_PATTERN");
  c->pattern_rows = !(pt && strcmp(pt, "warps") == 0);
  const char* p1 = getenv("GTGPU_P1");
  c->p1_dfloat = !(p1 && strcmp(p1, "fp64") == 0);
  const char* un = getenv("GTGPU_UNIFORM");
  c->uniform_geom = !(un && strcmp(un, "0") == 0);
  const char* irs = getenv("GTGPU_IR_STALL");
  if (irs) {
    double ratio = 0.0;
    int count = 0;
    if (sscanf(irs, "%lf,%d", &ratio, &count) == 2 && ratio > 0.0 && ratio < 1.0 && count >= 1 && count <= 100) {
      c->ir_stall_ratio = ratio;
      c->ir_stall_count = count;
    }
  }
  const char* ird = getenv("GTGPU_IR_DELTA");
  if (ird) {
    const double d = atof(ird);
    if (d > 1e-6 && d < 1.0) c->ir_delta = d;
  }
  const char* ln = getenv("GTGPU_SPMV_LANES");
  const int lanes = ln ? atoi(ln) : 0;
  c->spmv_lanes = (lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8) ? lanes : 0;
  cudaMemset(c->d_err, 0, sizeof(uint32_t));
  cudaDeviceSynchronize();
  *out = c;
  return GT_OK;
}

int gt_ctx_destroy(gt_ctx* c) {
  if (!c) return GT_ERR_INVALID;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->side) cudaStreamSynchronize(c->side);
  if (c->aux) cudaStreamSynchronize(c->aux);
  for (auto& kv : c->live) cudaFree(kv.first);
  for (auto& kv : c->pool) cudaFree(kv.second);
  cudaFree(c->d_err);
  cudaFreeHost(c->h_err);
  cudaFreeHost(c->h_scratch);
  cudaFreeHost(c->h_dscratch);
  for (auto& m : c->marks) cudaEventDestroy(m.second);
  for (auto e : c->spare_events) cudaEventDestroy(e);
  for (auto e : c->free_events) cudaEventDestroy(e);
  cudaStreamDestroy(c->own_stream);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->aux) cudaStreamDestroy(c->aux);
  delete c;
  return GT_OK;
}

const char* gt_last_error(const gt_ctx* c) { return c ? c->err.c_str() : "null context"; }

int gt_ctx_synchronize(gt_ctx* c) {
  if (!c) return GT_ERR_INVALID;
  GT_CUDA(c, cudaStreamSynchronize(c->stream));
  GT_CUDA(c, cudaStreamSynchronize(c->side));
  GT_CUDA(c, cudaStreamSynchronize(c->aux));
  return GT_OK;
}

int gt_ctx_set_stream(gt_ctx* c, void* stream) {
  if (!c) return GT_ERR_INVALID;
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return GT_OK;
}

int gt_ctx_fma_rate(gt_ctx* c, int precision, double* tflops) {
  if (!c || !tflops) return GT_ERR_INVALID;
  cudaSetDevice(c->device);
  if (precision == GT_FP64) return fma_rate<double>(c, 1 << 11, tflops);
  if (precision == GT_FP32) return fma_rate<float>(c, 1 << 14, tflops);
  return set_error(c, GT_ERR_INVALID, "precision must be GT_FP64 or GT_FP32");
}

int gt_ctx_barrier_probe(gt_ctx* c, int ctas, int missing, int64_t timeout_ns) {
  if (!c) return GT_ERR_INVALID;
  cudaSetDevice(c->device);
  return barrier_probe(c, ctas, missing, timeout_ns);
}

int gt_ctx_launch_count(gt_ctx* c, int64_t* launches) {
  if (!c || !launches) return GT_ERR_INVALID;
  *launches = c->launches;
  return GT_OK;
}

int gt_ctx_graph_launch_count(gt_ctx* c, int64_t* launches) {
  if (!c || !launches) return GT_ERR_INVALID;
  *launches = c->graph_launches;
  return GT_OK;
}

int gt_ctx_profile_begin(gt_ctx* c) {
  if (!c) return GT_ERR_INVALID;
  for (auto& m : c->marks) c->spare_events.push_back(m.second);
  c->marks.clear();
  c->prof = true;
  mark(c, "begin");
  return GT_OK;
}

int gt_ctx_profile_end(gt_ctx* c, int max, char* names, double* ms, int* count) {
  if (!c || !count) return GT_ERR_INVALID;
  mark(c, "end");
  c->prof = false;
  GT_CUDA(c, cudaStreamSynchronize(c->stream));
  int n = 0;
  for (size_t i = 1; i < c->marks.size() && n < max; i++, n++) {
    float t = 0.f;
    cudaEventElapsedTime(&t, c->marks[i - 1].second, c->marks[i].second);
    if (ms) ms[n] = t;
    if (names) {
      strncpy(names + 32 * n, c->marks[i].first.c_str(), 31);
      names[32 * n + 31] = 0;
    }
  }
  *count = n;
  return GT_OK;
}

int gt_ctx_trim(gt_ctx* c) {
  if (!c) return GT_ERR_INVALID;
  cudaSetDevice(c->device);
  pool_trim(c);
  return GT_OK;
}

int gt_ctx_memory(gt_ctx* c, int64_t* live, int64_t* pooled) {
  if (!c) return GT_ERR_INVALID;
  if (live) *live = c->live_bytes;
  if (pooled) *pooled = c->pooled_bytes;
  return GT_OK;
}

}  // extern "C"
