// gt_batch.cu -- many independent solves advanced by one set of launches.
//
// A batch holds n assembled scalar matrices (block size 1).  Their rows are
// cut into tiles of TR = 256 / G rows (G lanes per row); every launch of the
// batched Jacobi-PCG runs one CTA per tile of every instance, and the CTAs of
// instances that have converged return at once, so one launch advances all
// live instances by one step.  Each instance keeps its own CG scalars
// (alpha, beta, residual, done flag) on the device, and its dot products are
// reduced deterministically: each CTA writes its partial, the last CTA of
// the instance (one counter per instance) sums that instance's partials in
// tile order.  An instance's result is therefore bitwise the same whatever
// else is in the batch.  A chunk of BCHUNK iterations is captured once in a
// CUDA graph and replayed until no instance is live.  GT_SOLVE_IR runs the
// batched PCG in FP32 with per-instance FP64 reliable updates (true residual
// b - A64 x whenever an instance's FP32 residual fell tenfold).
#include <cmath>
#include <cstring>
#include <vector>

#include "gt_internal.cuh"

namespace gt {

constexpr int BT = 256;     // threads per CTA
constexpr int BCHUNK = 16;  // iterations per captured graph

struct BState {
  double rz, pq, rr, bb, alpha, beta, tol2;
  double rmax2, delta2, rzold;  // reliable updates (see k_brl_update)
  int32_t done, iters, maxit, upd, nupd, pad;
};

struct BInst {
  const int64_t* rowptr;
  const int32_t* colind;
  const double* v64;
  const float* v32;
  const int32_t* diag;  // position of the diagonal in each row
  int64_t nrows;
  int64_t off;          // offset of the instance in the concatenated vectors
  int32_t t0, nt;       // first tile, number of tiles
};

struct BatchImpl {
  Ctx* ctx = nullptr;
  int n = 0, G = 4, tile_rows = 64;
  int64_t ntot = 0, ntiles = 0;
  std::vector<Matrix*> mats;
  std::vector<BInst> h_inst;
  BInst* d_inst = nullptr;
  int32_t* d_tile_inst = nullptr;
  int64_t* d_tile_row0 = nullptr;
  uint32_t* d_counter = nullptr;  // one per instance, returns to 0 after each use
  int32_t* d_active = nullptr;
  int32_t* h_active = nullptr;    // pinned
};

template <class T>
__device__ __forceinline__ T bwarp_sum(T v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Per-instance sum of K values over the instance's CTAs: true in every
// thread of the instance's last CTA, with the totals in v.
template <int K, class A>
__device__ bool inst_reduce(A (&v)[K], double* partials, uint32_t* counter, const BInst& in, int t) {
  __shared__ A sred[K][BT / 32];
  __shared__ double tree[K][BT];
  __shared__ int s_flag;
  int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    A s = bwarp_sum(v[k]);
    if (lane == 0) sred[k][w] = s;
  }
  __syncthreads();
  if (tid == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      A s = (A)0;
      for (int i = 0; i < BT / 32; i++) s += sred[k][i];
      partials[(size_t)t * K + k] = (double)s;
    }
    __threadfence();
    unsigned prev = atomicInc(counter, (unsigned)in.nt - 1u);
    s_flag = prev == (unsigned)in.nt - 1u;
  }
  __syncthreads();
  if (!s_flag) return false;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double s = 0.0;
    for (int i = tid; i < in.nt; i += BT) s += __ldcg(&partials[(size_t)(in.t0 + i) * K + k]);
    tree[k][tid] = s;
  }
  __syncthreads();
  for (int o = BT / 2; o; o >>= 1) {
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

template <int G, class V, class X>
__device__ __forceinline__ X brow_dot(const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                      const V* __restrict__ val, const X* __restrict__ x, int64_t r, int gl) {
  X acc = (X)0;
  int64_t b = rp[r], e = rp[r + 1];
  int64_t k = b + gl;
  for (; k + G < e; k += 2 * G) {
    int32_t j0 = __ldg(ci + k), j1 = __ldg(ci + k + G);
    X a0 = (X)__ldg(val + k), a1 = (X)__ldg(val + k + G);
    acc = fma(a0, x[j0], acc);
    acc = fma(a1, x[j1], acc);
  }
  if (k < e) acc = fma((X)__ldg(val + k), x[__ldg(ci + k)], acc);
#pragma unroll
  for (int o = G >> 1; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return acc;
}

template <class X>
__device__ __forceinline__ const X* bvals(const BInst& in) {
  if constexpr (sizeof(X) == 8) return (const X*)in.v64;
  else return (const X*)in.v32;
}

// q = A p, p.q -> alpha
template <int G, class X>
__global__ void __launch_bounds__(BT) k_bcg_spmv(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                                                 const int64_t* __restrict__ trow0, const X* __restrict__ p,
                                                 X* __restrict__ q, BState* st, double* partials, uint32_t* ctr) {
  int t = blockIdx.x;
  int i = tinst[t];
  if (st[i].done) return;
  BInst in = insts[i];
  int grp = threadIdx.x / G, gl = threadIdx.x - grp * G;
  int64_t r = trow0[t] + grp;
  bool valid = r < in.nrows;
  int64_t rr = valid ? r : in.nrows - 1;
  const X* pi = p + in.off;
  X o = brow_dot<G, X, X>(in.rowptr, in.colind, bvals<X>(in), pi, rr, gl);
  X v[1] = {(X)0};
  if (gl == 0 && valid) {
    q[in.off + r] = o;
    v[0] = o * pi[r];
  }
  if (inst_reduce<1, X>(v, partials, ctr + i, in, t) && threadIdx.x == 0) {
    st[i].pq = (double)v[0];
    st[i].alpha = st[i].rz / (double)v[0];
  }
}

template <class X>
__global__ void __launch_bounds__(BT) k_bcg_update(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                                                   const int64_t* __restrict__ trow0, int tile_rows, X* __restrict__ x,
                                                   X* __restrict__ r, X* __restrict__ z, const X* __restrict__ p,
                                                   const X* __restrict__ q, const X* __restrict__ dinv, BState* st,
                                                   double* partials, uint32_t* ctr, int32_t* active) {
  int t = blockIdx.x;
  int i = tinst[t];
  if (st[i].done) return;
  BInst in = insts[i];
  X alpha = (X)st[i].alpha;
  X v[2] = {(X)0, (X)0};
  int64_t row = trow0[t] + threadIdx.x;
  if (threadIdx.x < tile_rows && row < in.nrows) {
    int64_t g = in.off + row;
    X ri = r[g] - alpha * q[g];
    x[g] += alpha * p[g];
    X zi = dinv[g] * ri;
    r[g] = ri;
    z[g] = zi;
    v[0] = ri * zi;
    v[1] = ri * ri;
  }
  if (inst_reduce<2, X>(v, partials, ctr + i, in, t) && threadIdx.x == 0) {
    double rz = (double)v[0], rr = (double)v[1];
    st[i].beta = rz / st[i].rz;
    st[i].rz = rz;
    st[i].rr = rr;
    st[i].iters += 1;
    if (rr <= st[i].tol2 || st[i].iters >= st[i].maxit || !(rr == rr)) {
      st[i].done = 1;
      atomicSub(active, 1);
    }
  }
}

template <class X>
__global__ void __launch_bounds__(BT) k_bcg_pupdate(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                                                    const int64_t* __restrict__ trow0, int tile_rows,
                                                    X* __restrict__ p, const X* __restrict__ z, const BState* st) {
  int t = blockIdx.x;
  int i = tinst[t];
  if (st[i].done) return;
  BInst in = insts[i];
  int64_t row = trow0[t] + threadIdx.x;
  if (threadIdx.x < tile_rows && row < in.nrows) {
    int64_t g = in.off + row;
    p[g] = z[g] + (X)st[i].beta * p[g];
  }
}

// start from x = 0: r = rhs, z = Dinv r, p = z; tolerance relative to ||rhs||
template <class X>
__global__ void __launch_bounds__(BT) k_bcg_init(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                                                 const int64_t* __restrict__ trow0, int tile_rows,
                                                 const X* __restrict__ rhs, X* __restrict__ x, X* __restrict__ r,
                                                 X* __restrict__ z, X* __restrict__ p, const X* __restrict__ dinv,
                                                 BState* st, double* partials, uint32_t* ctr, double rtol2, int maxit,
                                                 const int32_t* skip, int32_t* active) {
  int t = blockIdx.x;
  int i = tinst[t];
  BInst in = insts[i];
  X v[2] = {(X)0, (X)0};
  int64_t row = trow0[t] + threadIdx.x;
  if (threadIdx.x < tile_rows && row < in.nrows) {
    int64_t g = in.off + row;
    X ri = rhs[g];
    X zi = dinv[g] * ri;
    x[g] = (X)0;
    r[g] = ri;
    z[g] = zi;
    p[g] = zi;
    v[0] = ri * zi;
    v[1] = ri * ri;
  }
  if (inst_reduce<2, X>(v, partials, ctr + i, in, t) && threadIdx.x == 0) {
    st[i].rz = (double)v[0];
    st[i].rr = (double)v[1];
    st[i].bb = (double)v[1];
    st[i].tol2 = rtol2 * (double)v[1];
    st[i].iters = 0;
    st[i].maxit = maxit;
    st[i].beta = 0.0;
    bool d = (skip && skip[i]) || v[1] == 0.0;
    st[i].done = d;
    if (!d) atomicAdd(active, 1);
  }
}

// y = b - A x (FP64 values and vectors); per instance ||y||^2 and ||b||^2
template <int G>
__global__ void __launch_bounds__(BT) k_bresid64(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                                                 const int64_t* __restrict__ trow0, const double* __restrict__ b,
                                                 const double* __restrict__ x, double* __restrict__ y,
                                                 double* __restrict__ norms, double* partials, uint32_t* ctr) {
  int t = blockIdx.x;
  int i = tinst[t];
  BInst in = insts[i];
  int grp = threadIdx.x / G, gl = threadIdx.x - grp * G;
  int64_t r = trow0[t] + grp;
  bool valid = r < in.nrows;
  int64_t rr = valid ? r : in.nrows - 1;
  double o = brow_dot<G, double, double>(in.rowptr, in.colind, in.v64, x + in.off, rr, gl);
  double v[2] = {0.0, 0.0};
  if (gl == 0 && valid) {
    double bi = b[in.off + r];
    double yi = bi - o;
    y[in.off + r] = yi;
    v[0] = yi * yi;
    v[1] = bi * bi;
  }
  if (inst_reduce<2, double>(v, partials, ctr + i, in, t) && threadIdx.x == 0) {
    norms[2 * i] = v[0];
    norms[2 * i + 1] = v[1];
  }
}

// ---------------------------------------------------------------------------
// Batched CG with FP64 reliable updates (GT_SOLVE_FP64 with delta = 0,
// GT_SOLVE_IR in FP32 with delta = 0.1): per instance, the iteration runs on
// the correction xs since the last update; when the recurrence residual fell
// by delta (or claims convergence, or maxit is reached) x += xs and the FP64
// true residual b - A x replaces the recurrence residual; the direction p is
// then rebuilt from it.  Convergence is decided on the true residual.
// ---------------------------------------------------------------------------

// x = 0, xs = 0, r = (X) b, z = Dinv r, p = z; ||b||^2, tolerance
template <class X>
__global__ void __launch_bounds__(BT) k_brl_init(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                                                 const int64_t* __restrict__ trow0, int tile_rows,
                                                 const double* __restrict__ b, double* __restrict__ x,
                                                 X* __restrict__ xs, X* __restrict__ r, X* __restrict__ z,
                                                 X* __restrict__ p, const X* __restrict__ dinv, BState* st,
                                                 double* partials, uint32_t* ctr, double rtol2, double delta2,
                                                 int maxit, int32_t* active) {
  int t = blockIdx.x;
  int i = tinst[t];
  BInst in = insts[i];
  double v[2] = {0.0, 0.0};
  int64_t row = trow0[t] + threadIdx.x;
  if (threadIdx.x < tile_rows && row < in.nrows) {
    int64_t g = in.off + row;
    double bi = b[g];
    X rx = (X)bi;
    X zx = dinv[g] * rx;
    x[g] = 0.0;
    xs[g] = (X)0;
    r[g] = rx;
    z[g] = zx;
    p[g] = zx;
    v[0] = (double)rx * (double)zx;
    v[1] = bi * bi;
  }
  if (inst_reduce<2, double>(v, partials, ctr + i, in, t) && threadIdx.x == 0) {
    BState s{};
    s.rz = v[0];
    s.rr = v[1];
    s.bb = v[1];
    s.tol2 = rtol2 * v[1];
    s.rmax2 = v[1];
    s.delta2 = delta2;
    s.maxit = maxit;
    s.done = v[1] == 0.0;
    st[i] = s;
    if (!s.done) atomicAdd(active, 1);
  }
}

template <class X>
__global__ void __launch_bounds__(BT) k_brl_update(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                                                   const int64_t* __restrict__ trow0, int tile_rows, X* __restrict__ xs,
                                                   X* __restrict__ r, X* __restrict__ z, const X* __restrict__ p,
                                                   const X* __restrict__ q, const X* __restrict__ dinv, BState* st,
                                                   double* partials, uint32_t* ctr) {
  int t = blockIdx.x;
  int i = tinst[t];
  if (st[i].done) return;
  BInst in = insts[i];
  X alpha = (X)st[i].alpha;
  X v[2] = {(X)0, (X)0};
  int64_t row = trow0[t] + threadIdx.x;
  if (threadIdx.x < tile_rows && row < in.nrows) {
    int64_t g = in.off + row;
    X ri = r[g] - alpha * q[g];
    xs[g] += alpha * p[g];
    X zi = dinv[g] * ri;
    r[g] = ri;
    z[g] = zi;
    v[0] = ri * zi;
    v[1] = ri * ri;
  }
  if (inst_reduce<2, X>(v, partials, ctr + i, in, t) && threadIdx.x == 0) {
    double rz = (double)v[0], rr = (double)v[1];
    BState& s = st[i];
    s.rzold = s.rz;
    s.beta = rz / s.rz;
    s.rz = rz;
    s.rr = rr;
    s.iters += 1;
    if (rr <= s.tol2 || rr <= s.delta2 * s.rmax2 || s.iters >= s.maxit || !(rr == rr)) s.upd = 1;
  }
}

// x += xs, xs = 0 for the instances with an update due
template <class X>
__global__ void __launch_bounds__(BT) k_brl_xupdate(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                                                    const int64_t* __restrict__ trow0, int tile_rows,
                                                    double* __restrict__ x, X* __restrict__ xs, const BState* st) {
  int t = blockIdx.x;
  int i = tinst[t];
  if (st[i].done || !st[i].upd) return;
  BInst in = insts[i];
  int64_t row = trow0[t] + threadIdx.x;
  if (threadIdx.x < tile_rows && row < in.nrows) {
    int64_t g = in.off + row;
    x[g] += (double)xs[g];
    xs[g] = (X)0;
  }
}

// r64 = b - A64 x, r = (X) r64, z = Dinv r; true-residual convergence test
template <int G, class X>
__global__ void __launch_bounds__(BT) k_brl_resid(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                                                  const int64_t* __restrict__ trow0, const double* __restrict__ b,
                                                  const double* __restrict__ x, X* __restrict__ r, X* __restrict__ z,
                                                  const X* __restrict__ dinv, BState* st, double* partials,
                                                  uint32_t* ctr, int32_t* active) {
  int t = blockIdx.x;
  int i = tinst[t];
  if (st[i].done || !st[i].upd) return;
  BInst in = insts[i];
  int grp = threadIdx.x / G, gl = threadIdx.x - grp * G;
  int64_t row = trow0[t] + grp;
  bool valid = row < in.nrows;
  int64_t rr = valid ? row : in.nrows - 1;
  double o = brow_dot<G, double, double>(in.rowptr, in.colind, in.v64, x + in.off, rr, gl);
  double v[2] = {0.0, 0.0};
  if (gl == 0 && valid) {
    int64_t g = in.off + row;
    double ri = b[g] - o;
    X rx = (X)ri;
    X zx = dinv[g] * rx;
    r[g] = rx;
    z[g] = zx;
    v[0] = (double)rx * (double)zx;
    v[1] = ri * ri;
  }
  if (inst_reduce<2, double>(v, partials, ctr + i, in, t) && threadIdx.x == 0) {
    BState& s = st[i];
    s.beta = s.rzold != 0.0 ? v[0] / s.rzold : 0.0;
    s.rz = v[0];
    s.rr = v[1];
    s.nupd += 1;
    s.rmax2 = v[1];
    s.upd = 0;
    if (v[1] <= s.tol2 || s.iters >= s.maxit || !(v[1] == v[1])) {
      s.done = 1;
      atomicSub(active, 1);
    }
  }
}

template <class X>
__global__ void k_bdinv(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                        const int64_t* __restrict__ trow0, int tile_rows, X* __restrict__ dinv) {
  int t = blockIdx.x;
  BInst in = insts[tinst[t]];
  int64_t row = trow0[t] + threadIdx.x;
  if (threadIdx.x < tile_rows && row < in.nrows) {
    int64_t pos = in.rowptr[row] + in.diag[row];
    double d = in.v64 ? in.v64[pos] : (double)in.v32[pos];
    dinv[in.off + row] = (X)(1.0 / d);
  }
}

// rf = r / ||r|| (per instance, FP32)
__global__ void k_bscale(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                         const int64_t* __restrict__ trow0, int tile_rows, const double* __restrict__ r,
                         const double* __restrict__ norms, float* __restrict__ rf) {
  int t = blockIdx.x;
  int i = tinst[t];
  BInst in = insts[i];
  int64_t row = trow0[t] + threadIdx.x;
  if (threadIdx.x < tile_rows && row < in.nrows) {
    double n2 = norms[2 * i];
    double sc = n2 > 0.0 ? 1.0 / sqrt(n2) : 1.0;
    rf[in.off + row] = (float)(r[in.off + row] * sc);
  }
}

// x += ||r|| d for the instances that ran an inner solve
__global__ void k_baddscaled(const BInst* __restrict__ insts, const int32_t* __restrict__ tinst,
                             const int64_t* __restrict__ trow0, int tile_rows, double* __restrict__ x,
                             const float* __restrict__ d, const double* __restrict__ norms,
                             const int32_t* __restrict__ skip) {
  int t = blockIdx.x;
  int i = tinst[t];
  if (skip[i]) return;
  BInst in = insts[i];
  int64_t row = trow0[t] + threadIdx.x;
  if (threadIdx.x < tile_rows && row < in.nrows) x[in.off + row] += sqrt(norms[2 * i]) * (double)d[in.off + row];
}

}  // namespace gt

struct gt_batch : gt::BatchImpl {};

namespace gt {

static int build_tiles(gt_batch* B) {
  Ctx* ctx = B->ctx;
  int tr = BT / B->G;
  std::vector<int32_t> tinst;
  std::vector<int64_t> trow0;
  for (int i = 0; i < B->n; i++) {
    BInst& in = B->h_inst[i];
    in.t0 = (int32_t)tinst.size();
    int64_t nt = (in.nrows + tr - 1) / tr;
    if (nt < 1) nt = 1;
    for (int64_t k = 0; k < nt; k++) {
      tinst.push_back(i);
      trow0.push_back(k * tr);
    }
    in.nt = (int32_t)nt;
  }
  B->ntiles = (int64_t)tinst.size();
  B->tile_rows = tr;
  dfree(ctx, B->d_tile_inst);
  dfree(ctx, B->d_tile_row0);
  GT_TRY(dalloc(ctx, &B->d_tile_inst, B->ntiles));
  GT_TRY(dalloc(ctx, &B->d_tile_row0, B->ntiles));
  GT_TRY(copy_in(ctx, B->d_tile_inst, tinst.data(), B->ntiles));
  GT_TRY(copy_in(ctx, B->d_tile_row0, trow0.data(), B->ntiles));
  GT_TRY(copy_in(ctx, B->d_inst, B->h_inst.data(), B->n));
  GT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return GT_OK;
}

template <class X>
static void enqueue_iteration(gt_batch* B, X* x, X* r, X* z, X* p, X* q, const X* dinv, BState* st, double* partials) {
  Ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  unsigned g = (unsigned)B->ntiles;
  switch (B->G) {
    case 2: k_bcg_spmv<2, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, p, q, st, partials, B->d_counter); break;
    case 4: k_bcg_spmv<4, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, p, q, st, partials, B->d_counter); break;
    case 8: k_bcg_spmv<8, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, p, q, st, partials, B->d_counter); break;
    default: k_bcg_spmv<16, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, p, q, st, partials, B->d_counter); break;
  }
  k_bcg_update<X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, B->tile_rows, x, r, z, p, q,
                                               dinv, st, partials, B->d_counter, B->d_active);
  k_bcg_pupdate<X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, B->tile_rows, p, z, st);
}

// Captures BCHUNK iterations (enqueue() once per iteration) in a CUDA graph
// and replays it until no instance is live or maxit iterations ran.
template <class F>
static int run_chunks(gt_batch* B, int maxit, F&& enqueue) {
  Ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  GT_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int64_t l0 = ctx->launches;
  for (int k = 0; k < BCHUNK; k++) enqueue();
  int64_t per_chunk = ctx->launches - l0;
  cudaError_t ce = cudaStreamEndCapture(s, &graph);
  if (ce != cudaSuccess) return check_cuda(ctx, ce, "cudaStreamEndCapture");
  ce = cudaGraphInstantiate(&exec, graph, 0);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(graph);
    return check_cuda(ctx, ce, "cudaGraphInstantiate");
  }
  int status = GT_OK;
  ctx->launches -= per_chunk;  // counted per replay below
  for (int it = 0; it < maxit + BCHUNK; it += BCHUNK) {
    ce = cudaGraphLaunch(exec, s);
    if (ce != cudaSuccess) { status = check_cuda(ctx, ce, "cudaGraphLaunch"); break; }
    ctx->launches += per_chunk;
    cudaMemcpyAsync(B->h_active, B->d_active, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) { status = check_cuda(ctx, ce, "batched PCG"); break; }
    if (*B->h_active <= 0) break;
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  return status;
}

// batched PCG from x = 0 on values of type X; per-instance iteration counts
// and final recurrence residuals in hst
template <class X>
static int batch_pcg(gt_batch* B, const X* rhs, X* x, const X* dinv, double rtol, int maxit, const int32_t* skip,
                     BState* st, double* partials, std::vector<BState>& hst) {
  Ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  int64_t n = B->ntot;
  X *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
  GT_TRY(dalloc(ctx, &r, n));
  GT_TRY(dalloc(ctx, &z, n));
  GT_TRY(dalloc(ctx, &p, n));
  GT_TRY(dalloc(ctx, &q, n));
  GT_CUDA(ctx, cudaMemsetAsync(B->d_active, 0, sizeof(int32_t), s));
  k_bcg_init<X><<<GT_KC(ctx, (unsigned)B->ntiles), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0,
                                                               B->tile_rows, rhs, x, r, z, p, dinv, st, partials,
                                                               B->d_counter, rtol * rtol, maxit, skip, B->d_active);
  GT_LAUNCH(ctx, "k_bcg_init");
  int status = run_chunks(B, maxit, [&]() { enqueue_iteration<X>(B, x, r, z, p, q, dinv, st, partials); });
  hst.resize(B->n);
  if (status == GT_OK) {
    GT_CUDA(ctx, cudaMemcpyAsync(hst.data(), st, sizeof(BState) * B->n, cudaMemcpyDeviceToHost, s));
    GT_CUDA(ctx, cudaStreamSynchronize(s));
  }
  dfree(ctx, r);
  dfree(ctx, z);
  dfree(ctx, p);
  dfree(ctx, q);
  return status;
}

// batched CG with FP64 reliable updates from x = 0 (iteration in X)
template <class X>
static int batch_rpcg(gt_batch* B, const double* b, double* x, const X* dinv, double rtol, int maxit, double delta,
                      BState* st, double* partials, std::vector<BState>& hst) {
  Ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  int64_t n = B->ntot;
  unsigned g = (unsigned)B->ntiles;
  X *xs = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
  GT_TRY(dalloc(ctx, &xs, n));
  GT_TRY(dalloc(ctx, &r, n));
  GT_TRY(dalloc(ctx, &z, n));
  GT_TRY(dalloc(ctx, &p, n));
  GT_TRY(dalloc(ctx, &q, n));
  GT_CUDA(ctx, cudaMemsetAsync(B->d_active, 0, sizeof(int32_t), s));
  k_brl_init<X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, B->tile_rows, b, x, xs, r, z,
                                             p, dinv, st, partials, B->d_counter, rtol * rtol, delta * delta, maxit,
                                             B->d_active);
  GT_LAUNCH(ctx, "k_brl_init");
  auto iteration = [&]() {
    switch (B->G) {
      case 2: k_bcg_spmv<2, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, p, q, st, partials, B->d_counter); break;
      case 4: k_bcg_spmv<4, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, p, q, st, partials, B->d_counter); break;
      case 8: k_bcg_spmv<8, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, p, q, st, partials, B->d_counter); break;
      default: k_bcg_spmv<16, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, p, q, st, partials, B->d_counter); break;
    }
    k_brl_update<X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, B->tile_rows, xs, r, z, p, q,
                                                 dinv, st, partials, B->d_counter);
    k_brl_xupdate<X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, B->tile_rows, x, xs, st);
    switch (B->G) {
      case 2: k_brl_resid<2, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, b, x, r, z, dinv, st, partials, B->d_counter, B->d_active); break;
      case 4: k_brl_resid<4, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, b, x, r, z, dinv, st, partials, B->d_counter, B->d_active); break;
      case 8: k_brl_resid<8, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, b, x, r, z, dinv, st, partials, B->d_counter, B->d_active); break;
      default: k_brl_resid<16, X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, b, x, r, z, dinv, st, partials, B->d_counter, B->d_active); break;
    }
    k_bcg_pupdate<X><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, B->tile_rows, p, z, st);
  };
  int status = run_chunks(B, maxit, iteration);
  hst.resize(B->n);
  if (status == GT_OK) {
    GT_CUDA(ctx, cudaMemcpyAsync(hst.data(), st, sizeof(BState) * B->n, cudaMemcpyDeviceToHost, s));
    GT_CUDA(ctx, cudaStreamSynchronize(s));
  }
  dfree(ctx, xs);
  dfree(ctx, r);
  dfree(ctx, z);
  dfree(ctx, p);
  dfree(ctx, q);
  return status;
}

static int batch_resid(gt_batch* B, const double* b, const double* x, double* y, double* norms, double* partials) {
  Ctx* ctx = B->ctx;
  unsigned g = (unsigned)B->ntiles;
  cudaStream_t s = ctx->stream;
  switch (B->G) {
    case 2: k_bresid64<2><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, b, x, y, norms, partials, B->d_counter); break;
    case 4: k_bresid64<4><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, b, x, y, norms, partials, B->d_counter); break;
    case 8: k_bresid64<8><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, b, x, y, norms, partials, B->d_counter); break;
    default: k_bresid64<16><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, b, x, y, norms, partials, B->d_counter); break;
  }
  GT_LAUNCH(ctx, "k_bresid64");
  return GT_OK;
}

static int batch_solve(gt_batch* B, const double* b, double* x, double rtol, int maxit, int mode, gt_solve_info* infos) {
  Ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  int64_t n = B->ntot;
  int ni = B->n;
  unsigned g = (unsigned)B->ntiles;
  BState* st = nullptr;
  double *partials = nullptr, *norms = nullptr;
  int32_t* skip = nullptr;
  GT_TRY(dalloc(ctx, (unsigned char**)&st, (int64_t)sizeof(BState) * ni));
  GT_TRY(dalloc(ctx, &partials, 2 * B->ntiles + 2));
  GT_TRY(dalloc(ctx, &norms, 2 * (int64_t)ni));
  GT_TRY(dalloc(ctx, &skip, ni));
  GT_CUDA(ctx, cudaMemsetAsync(skip, 0, sizeof(int32_t) * ni, s));
  std::vector<gt_solve_info> info(ni);
  std::vector<BState> hst;
  int status = GT_OK;
  if (mode == GT_SOLVE_FP64 || mode == GT_SOLVE_FP32) {
    for (auto* A : B->mats)
      if ((mode == GT_SOLVE_FP64 && !A->val64) || (mode == GT_SOLVE_FP32 && !A->val32))
        return set_error(ctx, GT_ERR_INVALID, "batch solve: matrices lack the values of this mode");
  } else if (mode == GT_SOLVE_IR) {
    for (auto* A : B->mats)
      if (!A->val64 || !A->val32) return set_error(ctx, GT_ERR_INVALID, "batch IR solve needs GT_MIXED matrices");
  } else {
    return set_error(ctx, GT_ERR_INVALID, "unknown solve mode");
  }
  if (mode == GT_SOLVE_FP64) {
    double* dinv = nullptr;
    GT_TRY(dalloc(ctx, &dinv, n));
    k_bdinv<double><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, B->tile_rows, dinv);
    GT_LAUNCH(ctx, "k_bdinv");
    status = batch_rpcg<double>(B, b, x, dinv, rtol, maxit, 0.0, st, partials, hst);
    dfree(ctx, dinv);
    for (int i = 0; i < ni && status == GT_OK; i++) {
      info[i].iterations = hst[i].iters;
      info[i].outer_iterations = hst[i].nupd;
    }
  } else if (mode == GT_SOLVE_FP32) {
    float *dinv = nullptr, *bf = nullptr, *xf = nullptr;
    GT_TRY(dalloc(ctx, &dinv, n));
    GT_TRY(dalloc(ctx, &bf, n));
    GT_TRY(dalloc(ctx, &xf, n));
    k_bdinv<float><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, B->tile_rows, dinv);
    GT_CUDA(ctx, cudaMemsetAsync(norms, 0, sizeof(double) * 2 * ni, s));
    // rf = b (no scaling: norms = 0 -> factor 1)
    k_bscale<<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, B->tile_rows, b, norms, bf);
    GT_LAUNCH(ctx, "k_bscale");
    status = batch_pcg<float>(B, bf, xf, dinv, rtol, maxit, nullptr, st, partials, hst);
    GT_CUDA(ctx, cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    // x = xf: reuse k_baddscaled with norms[2i] = 1
    std::vector<double> ones(2 * ni, 1.0);
    GT_TRY(copy_in(ctx, norms, ones.data(), 2 * ni));
    k_baddscaled<<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, B->tile_rows, x, xf, norms,
                                              skip);
    GT_LAUNCH(ctx, "k_baddscaled");
    for (int i = 0; i < ni && status == GT_OK; i++) info[i].iterations = hst[i].iters;
    dfree(ctx, dinv);
    dfree(ctx, bf);
    dfree(ctx, xf);
  } else {
    // FP32 CG with FP64 reliable updates, per instance
    float* dinv = nullptr;
    GT_TRY(dalloc(ctx, &dinv, n));
    k_bdinv<float><<<GT_KC(ctx, g), BT, 0, s>>>(B->d_inst, B->d_tile_inst, B->d_tile_row0, B->tile_rows, dinv);
    GT_LAUNCH(ctx, "k_bdinv");
    status = batch_rpcg<float>(B, b, x, dinv, rtol, maxit, 0.1, st, partials, hst);
    dfree(ctx, dinv);
    for (int i = 0; i < ni && status == GT_OK; i++) {
      info[i].iterations = hst[i].iters;
      info[i].outer_iterations = hst[i].nupd;
    }
  }
  // true FP64 residuals where FP64 values exist (FP64 and IR modes)
  if (status == GT_OK && mode != GT_SOLVE_FP32) {
    double* r = nullptr;
    GT_TRY(dalloc(ctx, &r, n));
    GT_TRY(batch_resid(B, b, x, r, norms, partials));
    std::vector<double> hn(2 * ni);
    GT_CUDA(ctx, cudaMemcpyAsync(hn.data(), norms, sizeof(double) * 2 * ni, cudaMemcpyDeviceToHost, s));
    GT_CUDA(ctx, cudaStreamSynchronize(s));
    for (int i = 0; i < ni; i++) {
      info[i].rel_residual = hn[2 * i + 1] > 0 ? sqrt(hn[2 * i] / hn[2 * i + 1]) : 0.0;
      if (!(info[i].rel_residual <= rtol)) status = GT_ERR_NOT_CONVERGED;
    }
    dfree(ctx, r);
  }
  if (infos)
    for (int i = 0; i < ni; i++) infos[i] = info[i];
  pool_free(ctx, st);
  dfree(ctx, partials);
  dfree(ctx, norms);
  dfree(ctx, skip);
  if (status == GT_ERR_NOT_CONVERGED) set_error(ctx, status, "batch solve: some instance missed the tolerance");
  return status;
}

}  // namespace gt

using namespace gt;

extern "C" {

int gt_batch_create(gt_ctx* ctx, int n, gt_matrix* const* mats, gt_batch** out) {
  if (!ctx || !out || n <= 0 || !mats) return GT_ERR_INVALID;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  gt_batch* B = new gt_batch();
  B->ctx = ctx;
  B->n = n;
  int64_t off = 0;
  for (int i = 0; i < n; i++) {
    Matrix* A = mats[i];
    if (!A || A->ctx != ctx || A->bs != 1) {
      delete B;
      return set_error(ctx, GT_ERR_INVALID, "batch: matrices must be scalar (block size 1) and of this context");
    }
    int s = find_diag(A);
    if (s != GT_OK) {
      delete B;
      return s;
    }
    BInst in{};
    in.rowptr = A->rowptr;
    in.colind = A->colind;
    in.v64 = A->val64;
    in.v32 = A->val32;
    in.diag = A->diag_pos;
    in.nrows = A->nbrows;
    in.off = off;
    off += A->nbrows;
    B->h_inst.push_back(in);
    B->mats.push_back(A);
  }
  B->ntot = off;
  int s = dalloc(ctx, &B->d_inst, n);
  if (s == GT_OK) s = dalloc(ctx, &B->d_counter, n);
  if (s == GT_OK) s = dalloc(ctx, &B->d_active, 1);
  if (s == GT_OK && cudaMallocHost(&B->h_active, sizeof(int32_t)) != cudaSuccess) s = GT_ERR_CUDA;
  if (s == GT_OK && cudaMemsetAsync(B->d_counter, 0, sizeof(uint32_t) * n, ctx->stream) != cudaSuccess) s = GT_ERR_CUDA;
  if (s == GT_OK) s = build_tiles(B);
  if (s != GT_OK) {
    gt_batch_destroy(B);
    return s;
  }
  *out = B;
  return GT_OK;
}

int gt_batch_set_lanes(gt_batch* B, int lanes) {
  if (!B || (lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16)) return GT_ERR_INVALID;
  B->G = lanes;
  return build_tiles(B);
}

int gt_batch_info(const gt_batch* B, int64_t* info) {
  if (!B || !info) return GT_ERR_INVALID;
  info[0] = B->n;
  info[1] = B->ntot;
  info[2] = B->ntiles;
  info[3] = B->G;
  return GT_OK;
}

int gt_batch_solve(gt_batch* B, const double* b, double* x, double rtol, int maxit, int mode, gt_solve_info* infos) {
  if (!B || !b || !x) return GT_ERR_INVALID;
  Ctx* ctx = B->ctx;
  cudaSetDevice(ctx->device);
  cudaPointerAttributes ab{}, ax{};
  bool bdev = cudaPointerGetAttributes(&ab, b) == cudaSuccess && ab.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  bool xdev = cudaPointerGetAttributes(&ax, x) == cudaSuccess && ax.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  double *bd = (double*)b, *xd = x;
  if (!bdev) {
    GT_TRY(dalloc(ctx, &bd, B->ntot));
    GT_TRY(copy_in(ctx, bd, b, B->ntot));
  }
  if (!xdev) GT_TRY(dalloc(ctx, &xd, B->ntot));
  int s = batch_solve(B, bd, xd, rtol, maxit, mode, infos);
  if (!xdev) {
    int s2 = copy_out(ctx, x, xd, B->ntot);
    cudaStreamSynchronize(ctx->stream);
    if (s == GT_OK) s = s2;
    dfree(ctx, xd);
  }
  if (!bdev) dfree(ctx, bd);
  return s;
}

int gt_batch_destroy(gt_batch* B) {
  if (!B) return GT_ERR_INVALID;
  Ctx* ctx = B->ctx;
  dfree(ctx, B->d_inst);
  dfree(ctx, B->d_tile_inst);
  dfree(ctx, B->d_tile_row0);
  dfree(ctx, B->d_counter);
  dfree(ctx, B->d_active);
  if (B->h_active) cudaFreeHost(B->h_active);
  delete B;
  return GT_OK;
}

}  // extern "C"
