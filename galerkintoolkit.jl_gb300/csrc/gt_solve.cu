// gt_solve.cu -- block-CSR SpMV, Jacobi-preconditioned CG (FP64 and FP32)
// and FP64 iterative refinement around the FP32 CG.
//
// The reference has no iterative solver (it calls an external direct solve,
// src/problems.jl:439-462); this file is the GB300 replacement for that call.
//
// Every kernel runs one thread (vectors) or one lane group (SpMV rows) per
// item over a full grid, so all loads of a pass are in flight at once.  Dot
// products are reduced deterministically in two fixed levels: each CTA
// writes its partial, the last CTA of every group of 256 CTAs (threadfence +
// counter) sums the group in a fixed tree, and the last group sums the group
// partials.  The CG scalars (alpha, beta, residual, iteration count, done
// flag) live on the device, so iterations need no host round trip; the host
// polls the done flag once per chunk of iterations.  Results are bitwise
// reproducible and independent of co-running work.
#include <cmath>
#include <cstring>
#include <type_traits>

#include "gt_internal.cuh"
#include "gt_rowdot.cuh"

namespace gt {

constexpr int RED_T = 256;  // threads per CTA of the reduction kernels
constexpr int GROUP = 256;  // CTAs per first-level reduction group
constexpr unsigned kOneLevel = 2048;  // grids up to this size reduce in one level
constexpr int64_t kLoopUpdate = int64_t(1) << 22;  // vector length of the looping update kernels
constexpr int CHUNK = 16;   // CG iterations between host polls
constexpr int CG_STALLED = 1;  // internal status: the FP32 iteration stalled

// Programmatic dependent launch (sm_90 and later) for the kernels of a CG
// iteration: each is launched with programmatic stream serialisation, so its
// CTAs may be scheduled while its predecessor on the stream is still in its
// last-CTA reduction; it waits for that predecessor to complete (and its
// writes to be visible) before it touches any memory.  Every CTA of a
// reduction kernel lets the dependents launch once its own share is done.
// Without the launch attribute both instructions are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
static void launch_pdl(Ctx* ctx, void (*kern)(KArgs...), unsigned grid, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(GT_KC(ctx, grid));
  cfg.blockDim = dim3(RED_T);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// CHUNK iterations of a CG loop, captured once into a CUDA graph and
// replayed for every chunk: one graph launch instead of about five kernel
// launches per iteration (the programmatic-launch edges between the kernels
// are kept by the capture; every launch argument is a device pointer or a
// size fixed for the solve).  When the capture or the instantiation fails
// (e.g. on the legacy default stream), the chunk runs as direct launches.
struct ChunkGraph {
  cudaGraphExec_t exec = nullptr;
  bool tried = false;
  ChunkGraph() = default;
  ChunkGraph(const ChunkGraph&) = delete;
  ChunkGraph& operator=(const ChunkGraph&) = delete;
  ~ChunkGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
  template <class F>
  int run(Ctx* ctx, cudaStream_t s, F&& body) {
    if (!tried) {
      tried = true;
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const int rc = body();
        const cudaError_t e = cudaStreamEndCapture(s, &g);
        if (rc == GT_OK && e == cudaSuccess && g && cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) exec = nullptr;
        if (g) cudaGraphDestroy(g);
      }
      cudaGetLastError();  // a failed capture leaves its error here; the direct path follows
    }
    if (exec) {
      GT_CUDA(ctx, cudaGraphLaunch(exec, s));
      ctx->graph_launches++;
      return GT_OK;
    }
    return body();
  }
};

// device-resident CG state (one per solve)
struct CGState {
  double rz, pq, rr, bb, alpha, beta;
  double tol2;    // (rtol * ||b||)^2
  double rmax2;   // ||r||^2 at the last reliable update
  double delta2;  // reliable update when the recurrence residual fell by delta
  double rzold;   // r.z before the last recurrence step
  int32_t done;   // 1 converged or maxit, 2 FP32 iteration stalled or slowed down
  int32_t iters, maxit, upd, nupd;
  int32_t it_upd, max_cyc, stall, slow;  // reliable-update cycle bookkeeping
  double stall_ratio;   // hand-over rule (Ctx::ir_stall_ratio / ir_stall_count)
  int32_t stall_count, pad_;
};

// reduction scratch sized for the largest grid of a solve
struct RedBuf {
  double* p1;     // per-CTA partials (K per CTA)
  double* p2;     // per-group partials (K per group)
  uint32_t* ctr;  // group counters [ngroups] + final counter; each returns to 0 after use
};

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums K values over the whole grid.  Returns true in every thread of the one
// CTA that finishes last, with the totals in v; other CTAs return false.
// A: accumulator type of the in-CTA sums (the FP32 CG sums in FP32: GB300
// runs FP64 at 1/58 of the FP32 rate).  LEAD: only lanes that are multiples
// of LEAD hold values, so the warp sum skips the rounds below LEAD.
template <int K, class A = double, int LEAD = 1>
__device__ bool reduce_last(A (&v)[K], RedBuf rb) {
  __shared__ A sred[K][RED_T / 32];
  __shared__ double tree[K][RED_T];
  __shared__ int s_flag;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    A t = v[k];
#pragma unroll
    for (int o = 16; o >= LEAD; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) sred[k][w] = t;
  }
  __syncthreads();
  const unsigned nb = gridDim.x, b = blockIdx.x;
  if (nb <= kOneLevel) {
    // one level: every CTA posts its partials and takes a ticket (release);
    // the CTA with the last ticket (acquire) sums all partials in a fixed
    // order -- each thread a strided run of CTAs, then a butterfly per warp
    // and the warp totals in order.  One fence and one atomic per CTA and a
    // single round of partial loads: the two-level scheme's extra fence,
    // atomic and load round trips sat on the critical path of every
    // reduction kernel's last CTA.
    if (tid == 0) {
#pragma unroll
      for (int k = 0; k < K; k++) {
        A t = (A)0;
        for (int i = 0; i < nw; i++) t += sred[k][i];
        rb.p1[(size_t)b * K + k] = (double)t;
      }
      unsigned prev;
      asm volatile("atom.acq_rel.gpu.global.inc.u32 %0, [%1], %2;" : "=r"(prev) : "l"(rb.ctr), "r"(nb - 1) : "memory");
      s_flag = prev == nb - 1;
    }
    __syncthreads();
    if (!s_flag) return false;
#pragma unroll
    for (int k = 0; k < K; k++) {
      double t = 0.0;
      for (unsigned i = tid; i < nb; i += RED_T) t += __ldcg(&rb.p1[(size_t)i * K + k]);
      for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (lane == 0) tree[k][w] = t;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; k++) {
      double t = 0.0;
      for (int i = 0; i < nw; i++) t += tree[k][i];
      v[k] = (A)t;
    }
    __syncthreads();
    return true;
  }
  const unsigned ng = (nb + GROUP - 1) / GROUP, g = b / GROUP;
  const unsigned gs = min((unsigned)GROUP, nb - g * GROUP);
  if (tid == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      A t = (A)0;
      for (int i = 0; i < nw; i++) t += sred[k][i];
      rb.p1[(size_t)b * K + k] = (double)t;
    }
    __threadfence();
    unsigned prev = atomicInc(&rb.ctr[g], gs - 1);
    s_flag = prev == gs - 1;
  }
  __syncthreads();
  if (!s_flag) return false;
#pragma unroll
  for (int k = 0; k < K; k++) tree[k][tid] = tid < (int)gs ? __ldcg(&rb.p1[((size_t)g * GROUP + tid) * K + k]) : 0.0;
  __syncthreads();
  for (int o = RED_T / 2; o; o >>= 1) {
    if (tid < o)
#pragma unroll
      for (int k = 0; k < K; k++) tree[k][tid] += tree[k][tid + o];
    __syncthreads();
  }
  if (tid == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) rb.p2[(size_t)g * K + k] = tree[k][0];
    __threadfence();
    unsigned prev = atomicInc(&rb.ctr[ng], ng - 1);
    s_flag = prev == ng - 1;
  }
  __syncthreads();
  if (!s_flag) return false;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double t = 0.0;
    for (unsigned i = tid; i < ng; i += RED_T) t += __ldcg(&rb.p2[(size_t)i * K + k]);
    tree[k][tid] = t;
  }
  __syncthreads();
  for (int o = RED_T / 2; o; o >>= 1) {
    if (tid < o)
#pragma unroll
      for (int k = 0; k < K; k++) tree[k][tid] += tree[k][tid + o];
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < K; k++) v[k] = (A)tree[k][0];
  __syncthreads();
  return true;
}

// ---------------------------------------------------------------------------
// SpMV: G lanes per block row (row_dot, gt_rowdot.cuh); whole groups stay in
// the shuffles, rows past the end compute the last row again and write
// nothing
// ---------------------------------------------------------------------------
template <int BS, int G, class V, class X>
__device__ __forceinline__ void row_product(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                            const V* __restrict__ val, const X* __restrict__ x, int64_t r, int gl,
                                            X* out) {
  row_dot<BS, G, V, X, X, false>(rowptr, colind, val, x, r, gl, out);
}

// y = A x   (or y = bsub - A x)
template <int BS, int G, class V, class X>
__global__ void __launch_bounds__(RED_T) k_spmv(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                                const V* __restrict__ val, const X* __restrict__ x, int64_t nrows,
                                                const X* __restrict__ bsub, X* __restrict__ y) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t r = t / G;
  int gl = (int)(t - r * G);
  bool valid = r < nrows;
  if (!valid) r = nrows - 1;
  X o[BS];
  row_product<BS, G, V, X>(rowptr, colind, val, x, r, gl, o);
  if (gl == 0 && valid)
#pragma unroll
    for (int c = 0; c < BS; c++) y[r * BS + c] = bsub ? bsub[r * BS + c] - o[c] : o[c];
}

// q = A p and p.q; the last CTA sets alpha = rz / pq.  Each lane group
// handles RPG adjacent rows (independent loads in flight together; the CTA
// reduction is amortised over more rows).
constexpr int RPG = 2;
template <int BS, int G, class V, class X>
__global__ void __launch_bounds__(RED_T) k_cg_spmv(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                                   const V* __restrict__ val, const X* __restrict__ p, X* __restrict__ q,
                                                   int64_t nrows, CGState* st, RedBuf rb) {
  pdl_wait();
  if (st->done) return;
  X v[1] = {(X)0};
  // grid-stride with block-uniform trips (whole groups stay in the shuffles)
  const int64_t ngroups = (nrows + RPG - 1) / RPG;
  for (int64_t t0 = (int64_t)blockIdx.x * blockDim.x; t0 < ngroups * G; t0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = t0 + threadIdx.x;
    const int64_t grp = t / G;
    const int gl = (int)(t - grp * G);
#pragma unroll
    for (int u = 0; u < RPG; u++) {
      int64_t r = grp * RPG + u;
      bool valid = r < nrows;
      if (!valid) r = nrows - 1;
      X o[BS];
      row_product<BS, G, V, X>(rowptr, colind, val, p, r, gl, o);
      if (gl == 0 && valid) {
#pragma unroll
        for (int c = 0; c < BS; c++) {
          q[r * BS + c] = o[c];
          v[0] += o[c] * p[r * BS + c];
        }
      }
    }
  }
  pdl_release();
  if (reduce_last<1, X, G>(v, rb) && threadIdx.x == 0) {
    st->pq = (double)v[0];
    st->alpha = st->rz / (double)v[0];
  }
}

// x += alpha p; r -= alpha q; z = Dinv r; r.z and r.r -> beta, convergence.
// IPT elements per thread (coalesced, all loads issued before the math).
constexpr int IPT = 4;
template <class X, bool LOOP>
__global__ void __launch_bounds__(RED_T) k_cg_update(X* __restrict__ x, X* __restrict__ r, X* __restrict__ z,
                                                     const X* __restrict__ p, const X* __restrict__ q,
                                                     const X* __restrict__ dinv, int64_t n, CGState* st, RedBuf rb) {
  pdl_wait();
  if (st->done) return;
  const X alpha = (X)st->alpha;
  X v[2] = {(X)0, (X)0};
  auto trip = [&](const int64_t base) {
    X rv[IPT], qv[IPT], pv[IPT], xv[IPT], dv[IPT];
#pragma unroll
    for (int j = 0; j < IPT; j++) {
      int64_t i = base + (int64_t)j * blockDim.x;
      bool ok = i < n;
      rv[j] = ok ? r[i] : (X)0;
      qv[j] = ok ? q[i] : (X)0;
      pv[j] = ok ? p[i] : (X)0;
      xv[j] = ok ? x[i] : (X)0;
      dv[j] = ok ? dinv[i] : (X)0;
    }
#pragma unroll
    for (int j = 0; j < IPT; j++) {
      int64_t i = base + (int64_t)j * blockDim.x;
      X ri = rv[j] - alpha * qv[j];
      X zi = dv[j] * ri;
      if (i < n) {
        x[i] = xv[j] + alpha * pv[j];
        r[i] = ri;
        z[i] = zi;
      }
      v[0] += ri * zi;
      v[1] += ri * ri;
    }
  };
  if constexpr (LOOP) {
    // one wave of CTAs over the vector: fewer CTAs in the reduction
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x * IPT + threadIdx.x; base < n;
         base += (int64_t)gridDim.x * blockDim.x * IPT)
      trip(base);
  } else {
    trip((int64_t)blockIdx.x * blockDim.x * IPT + threadIdx.x);
  }
  pdl_release();
  if (reduce_last<2, X>(v, rb) && threadIdx.x == 0) {
    double rz = (double)v[0], rr = (double)v[1];
    st->beta = rz / st->rz;
    st->rz = rz;
    st->rr = rr;
    st->iters += 1;
    if (rr <= st->tol2 || st->iters >= st->maxit || !(rr == rr)) st->done = 1;
  }
}

template <class X>
__global__ void __launch_bounds__(RED_T) k_cg_pupdate(X* __restrict__ p, const X* __restrict__ z, int64_t n,
                                                      const CGState* st) {
  pdl_wait();
  if (st->done) return;
  const int64_t base = (int64_t)blockIdx.x * blockDim.x * IPT + threadIdx.x;
  const X beta = (X)st->beta;
  X zv[IPT], pv[IPT];
#pragma unroll
  for (int j = 0; j < IPT; j++) {
    int64_t i = base + (int64_t)j * blockDim.x;
    zv[j] = i < n ? z[i] : (X)0;
    pv[j] = i < n ? p[i] : (X)0;
  }
#pragma unroll
  for (int j = 0; j < IPT; j++) {
    int64_t i = base + (int64_t)j * blockDim.x;
    if (i < n) p[i] = zv[j] + beta * pv[j];
  }
}

// CG start: z = Dinv r; p = z; r.z and r.r; tolerance from ||b||^2 (or ||r0||^2)
template <class X>
__global__ void __launch_bounds__(RED_T) k_cg_init(const X* __restrict__ r, X* __restrict__ z, X* __restrict__ p,
                                                   const X* __restrict__ dinv, int64_t n, CGState* st, RedBuf rb,
                                                   double rtol2, const double* bb_dev) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double v[2] = {0.0, 0.0};
  if (i < n) {
    X zi = dinv[i] * r[i];
    z[i] = zi;
    p[i] = zi;
    v[0] = (double)r[i] * (double)zi;
    v[1] = (double)r[i] * (double)r[i];
  }
  if (reduce_last<2>(v, rb) && threadIdx.x == 0) {
    st->rz = v[0];
    st->rr = v[1];
    double ref = bb_dev ? *bb_dev : v[1];
    st->bb = ref;
    st->tol2 = rtol2 * ref;
    st->iters = 0;
    st->beta = 0.0;
    st->done = (v[1] <= st->tol2) || v[1] == 0.0;
  }
}

template <class X>
__global__ void __launch_bounds__(RED_T) k_norm2(const X* __restrict__ x, int64_t n, double* out, RedBuf rb) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double v[1] = {i < n ? (double)x[i] * (double)x[i] : 0.0};
  if (reduce_last<1>(v, rb) && threadIdx.x == 0) *out = v[0];
}

// Jacobi: dinv = 1 / diag(A) (per scalar row)
template <int BS, class V, class X>
__global__ void k_dinv(const int64_t* rowptr, const int32_t* diag_pos, const V* val, int64_t nbrows, X* dinv) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nbrows * BS) return;
  int64_t r = t / BS;
  int c = (int)(t - r * BS);
  int64_t k = rowptr[r] + diag_pos[r];
  dinv[t] = (X)(1.0 / (double)val[k * BS * BS + c * BS + c]);
}

__global__ void k_copy_f64_to_f32(const double* a, int64_t n, float* out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)a[i];
}
__global__ void k_copy_f32_to_f64(const float* a, int64_t n, double* out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)a[i];
}


// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// lanes per block row (row_lanes, gt_rowdot.cuh)
static int pick_group(const Matrix* A) {
  if (A->ctx->spmv_lanes) return A->ctx->spmv_lanes;
  return row_lanes(A->nbrows > 0 ? (double)A->bnnz / (double)A->nbrows : 1.0);
}
static unsigned spmv_grid(const Matrix* A) {
  int64_t g = (A->nbrows * pick_group(A) + RED_T - 1) / RED_T;
  return (unsigned)(g > 0 ? g : 1);
}
static unsigned cg_spmv_grid(const Matrix* A) {
  int64_t groups = (A->nbrows + RPG - 1) / RPG;
  int64_t g = (groups * pick_group(A) + RED_T - 1) / RED_T;
  return (unsigned)(g > 0 ? g : 1);
}
static unsigned ipt_grid(int64_t n) {
  int64_t g = (n + (int64_t)RED_T * IPT - 1) / ((int64_t)RED_T * IPT);
  return (unsigned)(g > 0 ? g : 1);
}
static unsigned vec_grid(int64_t n) {
  int64_t g = (n + RED_T - 1) / RED_T;
  return (unsigned)(g > 0 ? g : 1);
}
// One wave of a grid-stride kernel whose work is g CTA-sized trips: at most
// the CTAs of kern resident at once, and balanced -- T = ceil(g / cap) trips
// each for ceil(g / T) CTAs, so no CTA makes one trip more than most (with
// the plain cap, CTAs making two trips against others' one doubled the
// kernel's critical path).
template <class K>
static unsigned one_wave(const Ctx* ctx, K kern, unsigned g) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RED_T, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  const unsigned cap = (unsigned)per_sm * (unsigned)(ctx->num_sms > 0 ? ctx->num_sms : 1);
  if (g <= cap) return g > 0 ? g : 1;
  const unsigned trips = (g + cap - 1) / cap;
  return (g + trips - 1) / trips;
}
// grid-stride kernels that run at few iterations and exit at the others
static unsigned resident_grid(const Ctx* ctx, unsigned g) {
  const unsigned cap = 4u * (unsigned)(ctx->num_sms > 0 ? ctx->num_sms : 1);
  return g < cap ? g : cap;
}

// ---------------------------------------------------------------------------
// Sliced-ELL copy of a scalar matrix for the CG SpMV, built per solve.
// Slices of 32 consecutive rows, one lane per row; a slice stores its rows
// padded to its longest one, column-major (entry k of row 32 s + l at
// sptr[s] + 32 k + l; padding: the row's own column, value 0).  A warp then
// reads 32 rows' k-th column ids and values as two full 128-byte lines where
// the CSR row kernel issued 4-byte loads of lanes on different rows (whose
// load-queue occupancy, not DRAM, bounded the short P1/Q1 rows).  Each row
// is summed serially in column order.  Taken when the padding stays within
// a quarter of the entries.
// ---------------------------------------------------------------------------
constexpr int SELL_C = 32;

// view of a matrix's sliced copy in value type V (val == nullptr: not used)
template <class V>
struct SellView {
  int64_t nslices = 0;
  const int64_t* ptr = nullptr;
  const int32_t* len = nullptr;
  const int32_t* col = nullptr;
  const V* val = nullptr;
};

// warp per slice: the slice's longest row (and 32x it for the scan)
__global__ void k_sell_len(const int64_t* __restrict__ rowptr, int64_t nrows, int64_t nslices, int32_t* __restrict__ slen,
                           int32_t* __restrict__ slen32) {
  const int64_t sl = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (sl >= nslices) return;  // warp-uniform
  const int64_t r = sl * SELL_C + lane;
  int len = r < nrows ? (int)(rowptr[r + 1] - rowptr[r]) : 0;
  for (int o = 16; o; o >>= 1) len = max(len, __shfl_xor_sync(0xffffffffu, len, o));
  if (lane == 0) {
    slen[sl] = len;
    slen32[sl] = len * SELL_C;
  }
}

template <class V>
__global__ void k_sell_fill(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                            const V* __restrict__ val, int64_t nrows, int64_t nslices, const int64_t* __restrict__ sptr,
                            const int32_t* __restrict__ slen, int32_t* __restrict__ scol, V* __restrict__ sval) {
  const int64_t sl = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (sl >= nslices) return;
  const int64_t r = sl * SELL_C + lane;
  int64_t b = 0, e = 0;
  if (r < nrows) {
    b = rowptr[r];
    e = rowptr[r + 1];
  }
  const int32_t pad = r < nrows ? (int32_t)r : 0;
  const int L = slen[sl];
  const int64_t o = sptr[sl] + lane;
  for (int k = 0; k < L; k++) {
    const bool in = b + k < e;
    scol[o + (int64_t)k * SELL_C] = in ? colind[b + k] : pad;
    sval[o + (int64_t)k * SELL_C] = in ? val[b + k] : (V)0;
  }
}

// q = A p and p.q on the sliced copy; warp per slice, grid-stride over the
// slices (one wave), 4 entries per lane in flight
template <class V, class X>
__global__ void __launch_bounds__(RED_T) k_cg_spmv_sell(const int64_t* __restrict__ sptr, const int32_t* __restrict__ slen,
                                                        const int32_t* __restrict__ scol, const V* __restrict__ sval,
                                                        const X* __restrict__ p, X* __restrict__ q, int64_t nrows,
                                                        int64_t nslices, CGState* st, RedBuf rb) {
  pdl_wait();
  if (st->done) return;
  const int lane = threadIdx.x & 31;
  X v[1] = {(X)0};
  const int64_t wstride = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t sl = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; sl < nslices; sl += wstride) {
    const int64_t o = __ldg(sptr + sl) + lane;
    const int L = __ldg(slen + sl);
    X acc = (X)0;
    for (int k = 0; k < L; k += 4) {
      int32_t j[4];
      V a[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const bool in = k + u < L;
        j[u] = in ? __ldg(scol + o + (int64_t)(k + u) * SELL_C) : 0;
        a[u] = in ? __ldg(sval + o + (int64_t)(k + u) * SELL_C) : (V)0;
      }
      X xv[4];
#pragma unroll
      for (int u = 0; u < 4; u++) xv[u] = k + u < L ? p[j[u]] : (X)0;
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (k + u < L) acc = fma((X)a[u], xv[u], acc);
    }
    const int64_t r = sl * SELL_C + lane;
    if (r < nrows) {
      q[r] = acc;
      v[0] += acc * p[r];
    }
  }
  pdl_release();
  if (reduce_last<1, X>(v, rb) && threadIdx.x == 0) {
    st->pq = (double)v[0];
    st->alpha = st->rz / (double)v[0];
  }
}

template <class V>
static V*& sell_values(Matrix* A);
template <>
double*& sell_values<double>(Matrix* A) { return A->sell_v64; }
template <>
float*& sell_values<float>(Matrix* A) { return A->sell_v32; }
template <class V>
static bool& sell_current(Matrix* A);
template <>
bool& sell_current<double>(Matrix* A) { return A->sell_cur64; }
template <>
bool& sell_current<float>(Matrix* A) { return A->sell_cur32; }

void sell_release(Matrix* A) {
  Ctx* ctx = A->ctx;
  dfree(ctx, A->sell_ptr);
  dfree(ctx, A->sell_len);
  dfree(ctx, A->sell_col);
  dfree(ctx, A->sell_v64);
  dfree(ctx, A->sell_v32);
  A->sell_ptr = nullptr;
  A->sell_len = nullptr;
  A->sell_col = nullptr;
  A->sell_v64 = nullptr;
  A->sell_v32 = nullptr;
  A->sell_state = 0;
  A->sell_cur64 = A->sell_cur32 = false;
}

// The sliced copy of a scalar matrix with values val (A->val64 or A->val32),
// built on first use and refilled after value updates; view->val stays null
// when the copy does not apply (block rows, the opt-in tiled kernel, or a
// padding above a quarter of the entries -- then never retried).
template <class V>
static int sell_prepare(Matrix* A, const V* val, SellView<V>* view) {
  *view = SellView<V>{};
  Ctx* ctx = A->ctx;
  if (A->bs != 1 || A->nbrows == 0 || A->bnnz == 0 || A->sell_state < 0 || !val) return GT_OK;
  const int64_t nrows = A->nbrows, ns = (nrows + SELL_C - 1) / SELL_C;
  const unsigned g = (unsigned)((ns * 32 + 255) / 256);
  if (A->sell_state == 0) {
    int32_t* len32 = nullptr;
    GT_TRY(dalloc(ctx, &A->sell_len, ns));
    GT_TRY(dalloc(ctx, &A->sell_ptr, ns + 1));
    GT_TRY(dalloc(ctx, &len32, ns));
    k_sell_len<<<GT_KC(ctx, g), 256, 0, ctx->stream>>>(A->rowptr, nrows, ns, A->sell_len, len32);
    GT_LAUNCH(ctx, "k_sell_len");
    int st = exclusive_scan_i64(ctx, len32, A->sell_ptr, ns);
    dfree(ctx, len32);
    GT_TRY(st);
    GT_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scratch[4], A->sell_ptr + ns, sizeof(int64_t), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    GT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int64_t total = ctx->h_scratch[4];
    if (total > A->bnnz + A->bnnz / 4) {
      sell_release(A);
      A->sell_state = -1;
      return GT_OK;
    }
    GT_TRY(dalloc(ctx, &A->sell_col, total));
    A->sell_total = total;
    A->sell_nslices = ns;
    A->sell_state = 1;
    A->sell_cur64 = A->sell_cur32 = false;
  }
  V*& sv = sell_values<V>(A);
  if (!sv) GT_TRY(dalloc(ctx, &sv, A->sell_total));
  bool& cur = sell_current<V>(A);
  if (!cur) {
    k_sell_fill<V><<<GT_KC(ctx, g), 256, 0, ctx->stream>>>(A->rowptr, A->colind, val, nrows, ns, A->sell_ptr,
                                                           A->sell_len, A->sell_col, sv);
    GT_LAUNCH(ctx, "k_sell_fill");
    cur = true;
  }
  view->nslices = ns;
  view->ptr = A->sell_ptr;
  view->len = A->sell_len;
  view->col = A->sell_col;
  view->val = sv;
  return GT_OK;
}

// y = A x (or y = bsub - A x) on the sliced copy: warp per slice
template <class V, class X>
__global__ void k_spmv_sell(const int64_t* __restrict__ sptr, const int32_t* __restrict__ slen,
                            const int32_t* __restrict__ scol, const V* __restrict__ sval, const X* __restrict__ x,
                            int64_t nrows, int64_t nslices, const X* __restrict__ bsub, X* __restrict__ y) {
  const int64_t sl = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (sl >= nslices) return;
  const int64_t o = __ldg(sptr + sl) + lane;
  const int L = __ldg(slen + sl);
  X acc = (X)0;
  for (int k = 0; k < L; k += 4) {
    int32_t j[4];
    V a[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const bool in = k + u < L;
      j[u] = in ? __ldg(scol + o + (int64_t)(k + u) * SELL_C) : 0;
      a[u] = in ? __ldg(sval + o + (int64_t)(k + u) * SELL_C) : (V)0;
    }
    X xv[4];
#pragma unroll
    for (int u = 0; u < 4; u++) xv[u] = k + u < L ? x[j[u]] : (X)0;
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (k + u < L) acc = fma((X)a[u], xv[u], acc);
  }
  const int64_t r = sl * SELL_C + lane;
  if (r < nrows) y[r] = bsub ? bsub[r] - acc : acc;
}

struct Scratch {
  Ctx* ctx = nullptr;
  RedBuf rb{};
  int alloc(Ctx* c, unsigned max_grid) {
    ctx = c;
    unsigned ng = (max_grid + GROUP - 1) / GROUP;
    GT_TRY(dalloc(c, &rb.p1, (int64_t)max_grid * 2 + 2));
    GT_TRY(dalloc(c, &rb.p2, (int64_t)ng * 2 + 2));
    GT_TRY(dalloc(c, &rb.ctr, (int64_t)ng + 2));
    GT_CUDA(c, cudaMemsetAsync(rb.ctr, 0, sizeof(uint32_t) * (ng + 2), c->stream));
    return GT_OK;
  }
  ~Scratch() {
    if (ctx) {
      dfree(ctx, rb.p1);
      dfree(ctx, rb.p2);
      dfree(ctx, rb.ctr);
    }
  }
};

template <class V, class X>
struct Ops {
  template <class F>
  static void dispatch(int bs, int G, F&& go) {
    using I1 = std::integral_constant<int, 1>;
    using I2 = std::integral_constant<int, 2>;
    using I3 = std::integral_constant<int, 3>;
    auto byg = [&](auto bst) {
      if (G == 1) go(bst, std::integral_constant<int, 1>());
      else if (G == 2) go(bst, std::integral_constant<int, 2>());
      else if (G == 4) go(bst, std::integral_constant<int, 4>());
      else go(bst, std::integral_constant<int, 8>());
    };
    if (bs == 1) byg(I1());
    else if (bs == 2) byg(I2());
    else byg(I3());
  }
  static int spmv(Ctx* ctx, const Matrix* A, const V* val, const X* x, const X* bsub, X* y) {
    unsigned grid = spmv_grid(A);
    dispatch(A->bs, pick_group(A), [&](auto bs_t, auto g_t) {
      constexpr int BS = decltype(bs_t)::value, GG = decltype(g_t)::value;
      k_spmv<BS, GG, V, X><<<GT_KC(ctx, grid), RED_T, 0, ctx->stream>>>(A->rowptr, A->colind, val, x, A->nbrows, bsub, y);
    });
    GT_LAUNCH(ctx, "k_spmv");
    return GT_OK;
  }
  static int cg_spmv(Ctx* ctx, const Matrix* A, const V* val, const X* p, X* q, CGState* st, RedBuf rb,
                     const SellView<V>* sell = nullptr) {
    if (sell && sell->val) {
      auto kern = k_cg_spmv_sell<V, X>;
      const unsigned g = one_wave(ctx, kern, (unsigned)((sell->nslices * 32 + RED_T - 1) / RED_T));
      launch_pdl(ctx, kern, g, ctx->stream, sell->ptr, sell->len, sell->col, sell->val, p, q, A->nbrows,
                 sell->nslices, st, rb);
      GT_LAUNCH(ctx, "k_cg_spmv_sell");
      return GT_OK;
    }
    unsigned grid = cg_spmv_grid(A);
    dispatch(A->bs, pick_group(A), [&](auto bs_t, auto g_t) {
      constexpr int BS = decltype(bs_t)::value, GG = decltype(g_t)::value;
      launch_pdl(ctx, k_cg_spmv<BS, GG, V, X>, grid, ctx->stream, A->rowptr, A->colind, val, p, q, A->nbrows, st, rb);
    });
    GT_LAUNCH(ctx, "k_cg_spmv");
    return GT_OK;
  }
};

template <class X>
static int norm2(Ctx* ctx, const X* v, int64_t n, double* out_dev, RedBuf rb) {
  k_norm2<X><<<GT_KC(ctx, vec_grid(n)), RED_T, 0, ctx->stream>>>(v, n, out_dev, rb);
  GT_LAUNCH(ctx, "k_norm2");
  return GT_OK;
}

// PCG on A (values val) for A x = b; x holds the start value.  Vectors in X.
// The tolerance is relative to *bb_dev (||b||^2) or, if NULL, to ||r0||^2.
template <class V, class X>
static int pcg(Matrix* A, const V* val, const X* b, X* x, double rtol, int maxit, const double* bb_dev,
               int32_t* iters_out, double* rr_out, double* bb_out) {
  Ctx* ctx = A->space->mesh->ctx;
  cudaStream_t s = ctx->stream;
  int64_t n = A->nbrows * A->bs;
  X *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr;
  CGState* st = nullptr;
  unsigned gs = cg_spmv_grid(A), gv = vec_grid(n), gi = ipt_grid(n);
  Scratch sc;
  GT_TRY(sc.alloc(ctx, gs > gv ? gs : gv));
  GT_TRY(dalloc(ctx, &r, n));
  GT_TRY(dalloc(ctx, &z, n));
  GT_TRY(dalloc(ctx, &p, n));
  GT_TRY(dalloc(ctx, &q, n));
  GT_TRY(dalloc(ctx, &dinv, n));
  GT_TRY(dalloc(ctx, (unsigned char**)&st, sizeof(CGState)));
  CGState h0{};
  h0.maxit = maxit;
  GT_CUDA(ctx, cudaMemcpyAsync(st, &h0, sizeof(CGState), cudaMemcpyHostToDevice, s));
  GT_TRY(find_diag(A));
  if (A->bs == 1) k_dinv<1, V, X><<<GT_KC(ctx, grid_for(n, 256)), 256, 0, s>>>(A->rowptr, A->diag_pos, val, A->nbrows, dinv);
  else if (A->bs == 2) k_dinv<2, V, X><<<GT_KC(ctx, grid_for(n, 256)), 256, 0, s>>>(A->rowptr, A->diag_pos, val, A->nbrows, dinv);
  else k_dinv<3, V, X><<<GT_KC(ctx, grid_for(n, 256)), 256, 0, s>>>(A->rowptr, A->diag_pos, val, A->nbrows, dinv);
  GT_LAUNCH(ctx, "k_dinv");
  GT_TRY((Ops<V, X>::spmv(ctx, A, val, x, b, r)));  // r = b - A x
  k_cg_init<X><<<GT_KC(ctx, gv), RED_T, 0, s>>>(r, z, p, dinv, n, st, sc.rb, rtol * rtol, bb_dev);
  GT_LAUNCH(ctx, "k_cg_init");
  SellView<V> sell;
  GT_TRY(sell_prepare(A, val, &sell));
  // update kernel: up to kLoopUpdate elements, one wave of CTAs looping over
  // the vector (measured faster on 0.86M rows); above, one trip per thread
  // (the looping form holds twice the registers, which costs occupancy on
  // long vectors: measured slower on 19M rows)
  const bool uloop = n <= kLoopUpdate;
  const unsigned gu = uloop ? one_wave(ctx, k_cg_update<X, true>, gi) : gi;
  CGState h{};
  ChunkGraph graph;
  auto chunk = [&]() -> int {
    for (int k = 0; k < CHUNK; k++) {
      GT_TRY((Ops<V, X>::cg_spmv(ctx, A, val, p, q, st, sc.rb, &sell)));
      if (uloop) launch_pdl(ctx, k_cg_update<X, true>, gu, s, x, r, z, p, q, dinv, n, st, sc.rb);
      else launch_pdl(ctx, k_cg_update<X, false>, gu, s, x, r, z, p, q, dinv, n, st, sc.rb);
      launch_pdl(ctx, k_cg_pupdate<X>, gi, s, p, z, n, st);
    }
    GT_LAUNCH(ctx, "cg iteration");
    return GT_OK;
  };
  for (int it = 0; it < maxit; it += CHUNK) {
    GT_TRY(graph.run(ctx, s, chunk));
    GT_CUDA(ctx, cudaMemcpyAsync(ctx->h_dscratch, st, sizeof(CGState), cudaMemcpyDeviceToHost, s));
    GT_CUDA(ctx, cudaStreamSynchronize(s));
    memcpy(&h, ctx->h_dscratch, sizeof(CGState));
    if (h.done) break;
  }
  *iters_out = h.iters;
  *rr_out = h.rr;
  *bb_out = h.bb;
  int status = (h.rr <= h.tol2) ? GT_OK : GT_ERR_NOT_CONVERGED;
  dfree(ctx, r);
  dfree(ctx, z);
  dfree(ctx, p);
  dfree(ctx, q);
  dfree(ctx, dinv);
  pool_free(ctx, st);
  return status;
}

// ---------------------------------------------------------------------------
// CG with FP64 reliable updates.  The iteration runs in X (FP32 for the
// mixed mode, FP64 for the plain mode) on the correction xs since the last
// update; whenever the recurrence residual has dropped by delta (or claims
// convergence, or maxit is reached) the FP64 solution takes the correction
// (x += xs) and the FP64 true residual b - A x, computed with the FP64
// values, replaces the recurrence residual.  The search direction is kept,
// so the Krylov information survives the update and the iteration count
// stays near that of FP64 CG, at the per-iteration cost of X.  Convergence
// is declared on the FP64 true residual only.
// ---------------------------------------------------------------------------
template <class X, bool LOOP>
__global__ void __launch_bounds__(RED_T) k_rl_update(X* __restrict__ xs, X* __restrict__ r, X* __restrict__ z,
                                                     const X* __restrict__ p, const X* __restrict__ q,
                                                     const X* __restrict__ dinv, int64_t n, CGState* st, RedBuf rb) {
  pdl_wait();
  if (st->done) return;
  const X alpha = (X)st->alpha;
  X v[2] = {(X)0, (X)0};
  auto trip = [&](const int64_t base) {
    X rv[IPT], qv[IPT], pv[IPT], xv[IPT], dv[IPT];
#pragma unroll
    for (int j = 0; j < IPT; j++) {
      int64_t i = base + (int64_t)j * blockDim.x;
      bool ok = i < n;
      rv[j] = ok ? r[i] : (X)0;
      qv[j] = ok ? q[i] : (X)0;
      pv[j] = ok ? p[i] : (X)0;
      xv[j] = ok ? xs[i] : (X)0;
      dv[j] = ok ? dinv[i] : (X)0;
    }
#pragma unroll
    for (int j = 0; j < IPT; j++) {
      int64_t i = base + (int64_t)j * blockDim.x;
      X ri = rv[j] - alpha * qv[j];
      X zi = dv[j] * ri;
      if (i < n) {
        xs[i] = xv[j] + alpha * pv[j];
        r[i] = ri;
        z[i] = zi;
      }
      v[0] += ri * zi;
      v[1] += ri * ri;
    }
  };
  if constexpr (LOOP) {
    // one wave of CTAs over the vector: fewer CTAs in the reduction
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x * IPT + threadIdx.x; base < n;
         base += (int64_t)gridDim.x * blockDim.x * IPT)
      trip(base);
  } else {
    trip((int64_t)blockIdx.x * blockDim.x * IPT + threadIdx.x);
  }
  pdl_release();
  if (reduce_last<2, X>(v, rb) && threadIdx.x == 0) {
    double rz = (double)v[0], rr = (double)v[1];
    st->rzold = st->rz;
    st->beta = rz / st->rz;
    st->rz = rz;
    st->rr = rr;
    st->iters += 1;
    // an FP32 cycle running past 2.5x the longest earlier one: the FP32
    // iteration has lost the rate of the exact iteration (eps32 * cond(A))
    const int cyc = st->iters - st->it_upd;
    st->slow = sizeof(X) < sizeof(double) && (cyc > kSlowCycle || (st->max_cyc > 0 && cyc > (5 * st->max_cyc) / 2 + 16));
    if (rr <= st->tol2 || rr <= st->delta2 * st->rmax2 || st->iters >= st->maxit || !(rr == rr) || st->slow)
      st->upd = 1;
  }
}

// x += xs; xs = 0 (when an update is due).  Grid-stride over a grid of a
// few CTAs per SM: at the iterations without an update (nearly all) the
// launch costs only those CTAs reading the flag.
template <class X>
__global__ void __launch_bounds__(RED_T) k_rl_xupdate(double* __restrict__ x, X* __restrict__ xs, int64_t n,
                                                      const CGState* st) {
  pdl_wait();
  if (st->done || !st->upd) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += (double)xs[i];
    xs[i] = (X)0;
  }
}

// r64 = b - A x (FP64), r = (X) r64, z = Dinv r; rz and ||r64||^2; decides
// convergence on the true residual.  Grid-stride (block-uniform trips, so
// whole groups stay in row_dot's shuffles) over a grid of a few CTAs per SM,
// like k_rl_xupdate.
template <int BS, int G, class X>
__global__ void __launch_bounds__(RED_T) k_rl_resid(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                                    const double* __restrict__ val, const double* __restrict__ b,
                                                    const double* __restrict__ x, X* __restrict__ r, X* __restrict__ z,
                                                    const X* __restrict__ dinv, int64_t nrows, CGState* st, RedBuf rb) {
  pdl_wait();
  if (st->done || !st->upd) return;
  double v[2] = {0.0, 0.0};
  for (int64_t t0 = (int64_t)blockIdx.x * blockDim.x; t0 < nrows * G; t0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = t0 + threadIdx.x;
    int64_t row = t / G;
    const int gl = (int)(t - row * G);
    const bool valid = row < nrows;
    if (!valid) row = nrows - 1;
    double o[BS];
    row_product<BS, G, double, double>(rowptr, colind, val, x, row, gl, o);
    if (gl == 0 && valid) {
#pragma unroll
      for (int c = 0; c < BS; c++) {
        int64_t i = row * BS + c;
        double ri = b[i] - o[c];
        X rx = (X)ri;
        X zx = dinv[i] * rx;
        r[i] = rx;
        z[i] = zx;
        v[0] += (double)rx * (double)zx;
        v[1] += ri * ri;
      }
    }
  }
  pdl_release();
  if (reduce_last<2, double, G>(v, rb) && threadIdx.x == 0) {
    // the next direction is built from the true residual
    st->beta = st->rzold != 0.0 ? v[0] / st->rzold : 0.0;
    // the recurrence lost track of the true residual: restart the directions
    if (st->nupd > 0 && v[0] > (sizeof(X) == sizeof(double) ? kRestartRatio64 : kRestartRatio) * st->rz)
      st->beta = 0.0;
    const double prev = st->rmax2;
    st->rz = v[0];
    st->rr = v[1];
    st->nupd += 1;
    if (v[1] <= st->tol2 || st->iters >= st->maxit || !(v[1] == v[1])) st->done = 1;
    if (sizeof(X) == sizeof(double) && !st->done && st->nupd > 1) {
      // FP64: checks that do not halve ||r||, kStagnation times running: the
      // tolerance lies below the attainable accuracy; ends not converged
      st->stall = v[1] > 0.25 * prev ? st->stall + 1 : 0;
      if (st->stall >= kStagnation) st->done = 1;
    }
    if (sizeof(X) < sizeof(double) && !st->done && st->nupd > 1) {
      // the recurrence fell by delta but the true residual did not halve,
      // three times running, or the cycle slowed down: continue in FP64
      st->stall = v[1] > st->stall_ratio * prev ? st->stall + 1 : 0;
      if (st->stall >= st->stall_count || st->slow) st->done = 2;
    }
    const int cyc = st->iters - st->it_upd;
    if (st->nupd > 1 && cyc > st->max_cyc) st->max_cyc = cyc;
    st->it_upd = st->iters;
    st->rmax2 = v[1];
    st->upd = 0;
  }
}

template <class X>
__global__ void k_copy_vec(const X* __restrict__ a, X* __restrict__ out, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i];
}

__global__ void k_rl_setup(CGState* st, const double* bb, double rtol2, double delta2, int maxit, double stall_ratio,
                           int stall_count) {
  st->stall_ratio = stall_ratio;
  st->stall_count = stall_count;
  st->bb = *bb;
  st->tol2 = rtol2 * (*bb);
  st->delta2 = delta2;
  st->maxit = maxit;
  st->iters = 0;
  st->done = 0;
  st->upd = 1;
  st->nupd = 0;
  st->rmax2 = 1e300;
  st->beta = 0.0;
}

// Solve A x = b with CG in X plus FP64 reliable updates (see above); x (FP64)
// holds the start value on entry.  V: value type of the iteration's SpMV.
template <class V, class X>
static int pcg_reliable(Matrix* A, const V* val, const double* b, double* x, double rtol, int maxit, double delta,
                        int32_t* iters_out, int32_t* nupd_out, double* relres_out) {
  Ctx* ctx = A->space->mesh->ctx;
  cudaStream_t s = ctx->stream;
  int64_t n = A->nbrows * A->bs;
  X *xs = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr;
  CGState* st = nullptr;
  double* bb = nullptr;
  unsigned gs = cg_spmv_grid(A), gv = vec_grid(n), gi = ipt_grid(n), gr = spmv_grid(A);
  unsigned gmax = gs > gv ? gs : gv;
  if (gr > gmax) gmax = gr;
  Scratch sc;
  GT_TRY(sc.alloc(ctx, gmax));
  GT_TRY(dalloc(ctx, &xs, n));
  GT_TRY(dalloc(ctx, &r, n));
  GT_TRY(dalloc(ctx, &z, n));
  GT_TRY(dalloc(ctx, &p, n));
  GT_TRY(dalloc(ctx, &q, n));
  GT_TRY(dalloc(ctx, &dinv, n));
  GT_TRY(dalloc(ctx, &bb, 1));
  GT_TRY(dalloc(ctx, (unsigned char**)&st, sizeof(CGState)));
  GT_CUDA(ctx, cudaMemsetAsync(st, 0, sizeof(CGState), s));
  GT_CUDA(ctx, cudaMemsetAsync(xs, 0, sizeof(X) * n, s));
  GT_TRY(find_diag(A));
  if (A->bs == 1) k_dinv<1, double, X><<<GT_KC(ctx, grid_for(n, 256)), 256, 0, s>>>(A->rowptr, A->diag_pos, A->val64, A->nbrows, dinv);
  else if (A->bs == 2) k_dinv<2, double, X><<<GT_KC(ctx, grid_for(n, 256)), 256, 0, s>>>(A->rowptr, A->diag_pos, A->val64, A->nbrows, dinv);
  else k_dinv<3, double, X><<<GT_KC(ctx, grid_for(n, 256)), 256, 0, s>>>(A->rowptr, A->diag_pos, A->val64, A->nbrows, dinv);
  GT_LAUNCH(ctx, "k_dinv");
  GT_TRY(norm2(ctx, b, n, bb, sc.rb));
  k_rl_setup<<<GT_KC(ctx, 1), 1, 0, s>>>(st, bb, rtol * rtol, delta * delta, maxit, ctx->ir_stall_ratio,
                                         ctx->ir_stall_count);
  auto resid = [&]() {
    Ops<double, double>::dispatch(A->bs, pick_group(A), [&](auto bs_t, auto g_t) {
      constexpr int BS = decltype(bs_t)::value, GG = decltype(g_t)::value;
      launch_pdl(ctx, k_rl_resid<BS, GG, X>, resident_grid(ctx, gr), s, A->rowptr, A->colind, A->val64, b, x, r, z,
                 dinv, A->nbrows, st, sc.rb);
    });
  };
  resid();  // r = b - A x0, z, rz
  k_copy_vec<X><<<GT_KC(ctx, gv), RED_T, 0, s>>>(z, p, n);
  GT_LAUNCH(ctx, "reliable CG start");
  SellView<V> sell;
  GT_TRY(sell_prepare(A, val, &sell));
  // update kernel: up to kLoopUpdate elements, one wave of CTAs looping over
  // the vector (measured faster on 0.86M rows); above, one trip per thread
  // (the looping form holds twice the registers, which costs occupancy on
  // long vectors: measured slower on 19M rows)
  const bool uloop = n <= kLoopUpdate;
  const unsigned gu = uloop ? one_wave(ctx, k_rl_update<X, true>, gi) : gi;
  CGState h{};
  ChunkGraph graph;
  auto chunk = [&]() -> int {
    for (int k = 0; k < CHUNK; k++) {
      GT_TRY((Ops<V, X>::cg_spmv(ctx, A, val, p, q, st, sc.rb, &sell)));
      if (uloop) launch_pdl(ctx, k_rl_update<X, true>, gu, s, xs, r, z, p, q, dinv, n, st, sc.rb);
      else launch_pdl(ctx, k_rl_update<X, false>, gu, s, xs, r, z, p, q, dinv, n, st, sc.rb);
      launch_pdl(ctx, k_rl_xupdate<X>, resident_grid(ctx, gv), s, x, xs, n, st);
      resid();
      launch_pdl(ctx, k_cg_pupdate<X>, gi, s, p, z, n, st);
    }
    GT_LAUNCH(ctx, "reliable CG iteration");
    return GT_OK;
  };
  for (int it = 0; it < maxit + CHUNK; it += CHUNK) {
    GT_TRY(graph.run(ctx, s, chunk));
    GT_CUDA(ctx, cudaMemcpyAsync(ctx->h_dscratch, st, sizeof(CGState), cudaMemcpyDeviceToHost, s));
    GT_CUDA(ctx, cudaStreamSynchronize(s));
    memcpy(&h, ctx->h_dscratch, sizeof(CGState));
    if (h.done) break;
  }
  *iters_out = h.iters;
  *nupd_out = h.nupd;
  *relres_out = h.bb > 0 ? sqrt(h.rr / h.bb) : 0.0;
  int status = h.done == 2 ? CG_STALLED : (h.rr <= h.tol2) ? GT_OK : GT_ERR_NOT_CONVERGED;
  dfree(ctx, xs);
  dfree(ctx, r);
  dfree(ctx, z);
  dfree(ctx, p);
  dfree(ctx, q);
  dfree(ctx, dinv);
  dfree(ctx, bb);
  pool_free(ctx, st);
  return status;
}

int spmv64(Matrix* A, const double* x, double* y) {
  Ctx* ctx = A->space->mesh->ctx;
  if (!A->val64) return set_error(ctx, GT_ERR_INVALID, "matrix has no FP64 values");
  mark(ctx, "spmv_setup");
  SellView<double> sv;
  int s = sell_prepare(A, A->val64, &sv);  // first call: builds the sliced copy
  mark(ctx, "spmv_prepare");
  if (s == GT_OK && sv.val) {
    const unsigned g = (unsigned)((sv.nslices * 32 + 255) / 256);
    k_spmv_sell<double, double><<<GT_KC(ctx, g), 256, 0, ctx->stream>>>(sv.ptr, sv.len, sv.col, sv.val, x, A->nbrows,
                                                                        sv.nslices, nullptr, y);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) s = check_cuda(ctx, e, "k_spmv_sell");
  } else if (s == GT_OK) {
    s = Ops<double, double>::spmv(ctx, A, A->val64, x, nullptr, y);
  }
  mark(ctx, "spmv");  // the phase "spmv" of a profile is the kernel alone
  return s;
}

// ||b - A x|| / ||b|| in FP64
static int true_residual(Matrix* A, const double* b, const double* x, double* relres) {
  Ctx* ctx = A->space->mesh->ctx;
  int64_t n = A->nbrows * A->bs;
  double *r = nullptr, *scal = nullptr;
  Scratch sc;
  GT_TRY(sc.alloc(ctx, vec_grid(n)));
  GT_TRY(dalloc(ctx, &r, n));
  GT_TRY(dalloc(ctx, &scal, 2));
  GT_TRY((Ops<double, double>::spmv(ctx, A, A->val64, x, b, r)));
  GT_TRY(norm2(ctx, (const double*)r, n, scal, sc.rb));
  GT_TRY(norm2(ctx, b, n, scal + 1, sc.rb));
  GT_CUDA(ctx, cudaMemcpyAsync(ctx->h_dscratch, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  GT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double rn2 = ctx->h_dscratch[0], bn2 = ctx->h_dscratch[1];
  *relres = bn2 > 0 ? sqrt(rn2 / bn2) : 0.0;
  dfree(ctx, r);
  dfree(ctx, scal);
  return GT_OK;
}

int solve(Matrix* A, const double* b, double* x, double rtol, int maxit, int mode, gt_solve_info* info) {
  Ctx* ctx = A->space->mesh->ctx;
  cudaStream_t s = ctx->stream;
  int64_t n = A->nbrows * A->bs;
  gt_solve_info inf{};
  int status = GT_OK;
  if (n == 0) {
    if (info) *info = inf;
    return GT_OK;
  }
  unsigned gv = vec_grid(n);
  if (mode == GT_SOLVE_FP64 && !A->val64)
    return set_error(ctx, GT_ERR_INVALID, "GT_SOLVE_FP64 needs FP64 values (assemble with GT_FP64 or GT_MIXED)");
  if (mode == GT_SOLVE_FP32 && !A->val32)
    return set_error(ctx, GT_ERR_INVALID, "GT_SOLVE_FP32 needs FP32 values (GT_FP32 or GT_MIXED)");
  if (mode == GT_SOLVE_IR && (!A->val64 || !A->val32))
    return set_error(ctx, GT_ERR_INVALID, "GT_SOLVE_IR needs GT_MIXED values");
  if (mode != GT_SOLVE_FP64 && mode != GT_SOLVE_FP32 && mode != GT_SOLVE_IR)
    return set_error(ctx, GT_ERR_INVALID, "unknown solve mode");
  // the persistent kernel saves the per-phase launches and grid-wide
  // reduction tails that dominate small systems; large systems keep more
  // loads in flight with one launch per phase (measured crossover)
  const bool persistent = ctx->pcg_path == 2 || (ctx->pcg_path == 0 && n <= kPersistentMaxRows);
  if (persistent) {
    int32_t it = 0, nupd = 0, it64 = 0;
    status = pcg_persistent(A, mode, b, x, rtol, maxit, &it, &nupd, &it64, &inf.rel_residual);
    if (status != GT_OK && status != GT_ERR_NOT_CONVERGED) return status;
    inf.iterations = it;
    inf.outer_iterations = mode == GT_SOLVE_FP32 ? 0 : nupd;
    inf.fp64_iterations = it64;
    if (mode == GT_SOLVE_FP32 && A->val64) GT_TRY(true_residual(A, b, x, &inf.rel_residual));
    if (info) *info = inf;
    if (status == GT_ERR_NOT_CONVERGED) set_error(ctx, status, "solver did not reach the tolerance within maxit");
    return status;
  }
  if (mode == GT_SOLVE_FP64) {
    // FP64 CG; a recurrence residual below the tolerance is checked against
    // the true residual (delta = 0: updates only there) and the iteration
    // goes on from the true residual when that is still above it
    int32_t it = 0, nupd = 0;
    status = pcg_reliable<double, double>(A, A->val64, b, x, rtol, maxit, 0.0, &it, &nupd, &inf.rel_residual);
    inf.iterations = it;
    inf.outer_iterations = nupd;
    inf.fp64_iterations = it;
  } else if (mode == GT_SOLVE_FP32) {
    if (!A->val32) return set_error(ctx, GT_ERR_INVALID, "GT_SOLVE_FP32 needs FP32 values (GT_FP32 or GT_MIXED)");
    float *bf = nullptr, *xf = nullptr;
    GT_TRY(dalloc(ctx, &bf, n));
    GT_TRY(dalloc(ctx, &xf, n));
    k_copy_f64_to_f32<<<GT_KC(ctx, gv), RED_T, 0, s>>>(b, n, bf);
    k_copy_f64_to_f32<<<GT_KC(ctx, gv), RED_T, 0, s>>>(x, n, xf);
    GT_LAUNCH(ctx, "k_copy_f64_to_f32");
    int32_t it = 0;
    double rr = 0, bb = 0;
    status = pcg<float, float>(A, A->val32, bf, xf, rtol, maxit, nullptr, &it, &rr, &bb);
    k_copy_f32_to_f64<<<GT_KC(ctx, gv), RED_T, 0, s>>>(xf, n, x);
    GT_LAUNCH(ctx, "k_copy_f32_to_f64");
    inf.iterations = it;
    inf.rel_residual = bb > 0 ? sqrt(rr / bb) : 0.0;
    if (A->val64) GT_TRY(true_residual(A, b, x, &inf.rel_residual));
    dfree(ctx, bf);
    dfree(ctx, xf);
  } else if (mode == GT_SOLVE_IR) {
    if (!A->val64 || !A->val32) return set_error(ctx, GT_ERR_INVALID, "GT_SOLVE_IR needs GT_MIXED values");
    // FP32 CG (FP32 values, vectors and inner sums) with an FP64 true
    // residual and solution update each time the residual fell tenfold
    int32_t it = 0, nupd = 0;
    status = pcg_reliable<float, float>(A, A->val32, b, x, rtol, maxit, A->ctx->ir_delta, &it, &nupd, &inf.rel_residual);
    if (status == CG_STALLED) {
      // eps32 * cond(A) too large for the FP32 iteration: FP64 CG from the
      // current FP64 solution
      int32_t it2 = 0, nu2 = 0;
      status = pcg_reliable<double, double>(A, A->val64, b, x, rtol, maxit - it, 0.0, &it2, &nu2, &inf.rel_residual);
      inf.fp64_iterations = it2;
      it += it2;
      nupd += nu2;
    }
    inf.iterations = it;
    inf.outer_iterations = nupd;
  } else {
    return set_error(ctx, GT_ERR_INVALID, "unknown solve mode");
  }
  if (info) *info = inf;
  uint32_t bits = 0;
  GT_TRY(take_device_error(ctx, &bits));
  if (status == GT_ERR_NOT_CONVERGED) set_error(ctx, status, "solver did not reach the tolerance within maxit");
  return status;
}

}  // namespace gt

using namespace gt;

extern "C" {

int gt_solve(gt_matrix* A, const double* b, double* x, double rtol, int maxit, int mode, gt_solve_info* info) {
  if (!A || !b || !x) return GT_ERR_INVALID;
  Ctx* ctx = A->space->mesh->ctx;
  cudaSetDevice(ctx->device);
  int64_t n = A->nbrows * A->bs;
  cudaPointerAttributes ab{}, ax{};
  bool bdev = cudaPointerGetAttributes(&ab, b) == cudaSuccess && ab.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  bool xdev = cudaPointerGetAttributes(&ax, x) == cudaSuccess && ax.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  double *bd = (double*)b, *xd = x;
  if (!bdev) {
    GT_TRY(dalloc(ctx, &bd, n));
    GT_TRY(copy_in(ctx, bd, b, n));
  }
  if (!xdev) {
    GT_TRY(dalloc(ctx, &xd, n));
    GT_TRY(copy_in(ctx, xd, (const double*)x, n));
  }
  int s = solve(A, bd, xd, rtol, maxit, mode, info);
  if (!xdev) {
    int s2 = copy_out(ctx, x, xd, n);
    cudaStreamSynchronize(ctx->stream);
    if (s == GT_OK) s = s2;
    dfree(ctx, xd);
  }
  if (!bdev) dfree(ctx, bd);
  return s;
}

int gt_spmv(gt_matrix* A, const double* x, double* y) {
  if (!A || !x || !y) return GT_ERR_INVALID;
  Ctx* ctx = A->space->mesh->ctx;
  int64_t n = A->nbrows * A->bs;
  cudaPointerAttributes ax{}, ay{};
  bool xdev = cudaPointerGetAttributes(&ax, x) == cudaSuccess && ax.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  bool ydev = cudaPointerGetAttributes(&ay, y) == cudaSuccess && ay.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  double *xd = (double*)x, *yd = y;
  if (!xdev) {
    GT_TRY(dalloc(ctx, &xd, n));
    GT_TRY(copy_in(ctx, xd, x, n));
  }
  if (!ydev) GT_TRY(dalloc(ctx, &yd, n));
  int s = n > 0 ? spmv64(A, xd, yd) : GT_OK;
  if (s == GT_OK && !ydev) s = copy_out(ctx, y, yd, n);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (s == GT_OK && e != cudaSuccess) s = check_cuda(ctx, e, "gt_spmv");
  uint32_t bits = 0;
  if (s == GT_OK) s = take_device_error(ctx, &bits);
  if (!xdev) dfree(ctx, xd);
  if (!ydev) dfree(ctx, yd);
  return s;
}

}  // extern "C"
