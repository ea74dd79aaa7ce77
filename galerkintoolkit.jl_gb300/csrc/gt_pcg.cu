// gt_pcg.cu -- Jacobi-PCG as one persistent, cooperative kernel.
//
// The whole iteration runs inside one cooperative launch (chunks of
// iterations per launch): CTA c owns a contiguous range of block rows, every
// phase works on the CTA's own rows, and phases are separated by a grid-wide
// barrier.  A reduction is two-level and identical in every CTA: each CTA
// writes its partial sums, and after the barrier every CTA adds all partials
// in the same fixed order, so alpha, beta and the convergence decisions are
// bitwise the same in all CTAs without a further broadcast.  Per iteration:
//
//   P1  q = A p (own rows), p.q            -> barrier, alpha = rz / pq
//   P2  xs += alpha p, r -= alpha q,       -> barrier, beta, convergence
//       z = Dinv r, r.z, r.r
//   [reliable update, when due]
//   P3  x += xs, xs = 0                    -> barrier
//   P4  r = b - A64 x (FP64), z = Dinv r   -> barrier, r.z, ||r||^2
//   P5  p = z + beta p                     -> barrier
//
// The iteration runs in X (FP64 or FP32) on the correction xs since the last
// update, with SpMV values of type V.  With reliable updates (RELIABLE) the
// FP64 solution takes the correction and the FP64 true residual replaces the
// recurrence residual whenever the recurrence residual fell by delta since
// the last update, claims convergence, or maxit is reached; the direction p
// is then rebuilt from the true residual.  Convergence is decided on the
// FP64 true residual.  Without reliable updates (the FP32-only mode) the
// recurrence residual decides and x takes xs at the end.
//
// Every grid barrier waits with a time limit: a barrier that does not
// complete within a second records an error and the kernel returns (the
// cooperative launch makes all CTAs co-resident, so this does not happen in
// a correct run).
#include <cmath>
#include <cstring>

#include "gt_internal.cuh"
#include "gt_rowdot.cuh"

namespace gt {

namespace {

constexpr int PT = 256;          // threads per CTA
constexpr int NW = PT / 32;      // warps per CTA
constexpr int PSLOT = 4;         // doubles per CTA partial
constexpr uint64_t BAR_TIMEOUT_NS = 1000000000ull;
constexpr int PCG_STALLED = 1;   // internal status: the FP32 iteration stalled

struct PState {
  double rz, rzold, rr, rmax2, bb, tol2;
  int32_t iters, nupd;
  int32_t done;     // 1 converged or maxit, 2 FP32 iteration stalled or slowed down: continue in FP64
  int32_t stall;    // consecutive reliable updates with less than a halving of the true residual
  int32_t it_upd;   // iteration of the last reliable update
  int32_t max_cyc;  // longest cycle between reliable updates so far
};

struct PArgs {
  const int64_t* rowptr;
  const int32_t* colind;
  const void* val;       // iteration values (V)
  const double* val64;   // FP64 values (true residual), may be null without reliable updates
  int64_t nrows;         // block rows
  int nb;                // CTAs that solve this system (the grouped launch)
  const double* b;
  double* x;
  void *xs, *r, *z, *p, *q;
  const void* dinv;
  const float* pcont;    // FP32 direction to continue from (init mode 2)
  double* part;          // 3 slots x gridDim.x x PSLOT
  uint32_t* bar;         // barrier counter, zero at launch
  int32_t* err;          // set to 1 when a barrier timed out
  PState* st;
  double rtol2, delta2;
  int maxit;
  double stall_ratio;  // hand-over rule (Ctx::ir_stall_ratio / ir_stall_count)
  int stall_count;
};

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// grid-wide barrier number `target / gridDim.x`; false when it timed out
// (no arrival for timeout_ns: the error word is set and every CTA returns)
__device__ __forceinline__ bool grid_sync(uint32_t* bar, uint32_t target, int32_t* err, int* s_abort,
                                          uint64_t timeout_ns = BAR_TIMEOUT_NS) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
    uint64_t t0 = global_ns();
    while (ld_acquire(bar) < target) {
      if (global_ns() - t0 > timeout_ns) {
        atomicExch(err, 1);
        *s_abort = 1;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
  }
  __syncthreads();
  return *s_abort == 0;
}

// CTA sum of K values -> out[0..K) (written by thread 0)
template <int K>
__device__ __forceinline__ void cta_sum(double (&v)[K], double* s_red, double* out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double t = v[k];
#pragma unroll
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) s_red[k * NW + w] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      double t = 0.0;
#pragma unroll
      for (int i = 0; i < NW; i++) t += s_red[k * NW + i];
      __stcg(out + k, t);
    }
  }
}

// sum of the CTA partials of a slot, in one fixed order that is identical in
// every CTA: each thread loads its (at most a few) partials at once, warp
// butterflies (whose result is the same in all lanes), then the warp totals
// in warp order; result in s_tot[0..K).  s_red is free again at this point.
template <int K>
__device__ __forceinline__ void grid_total(const double* slot, int nb, double* s_red, double* s_tot) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double t[K];
#pragma unroll
  for (int k = 0; k < K; k++) t[k] = 0.0;
  for (int i = threadIdx.x; i < nb; i += PT) {
    const double2 v01 = __ldcg(reinterpret_cast<const double2*>(slot + (size_t)i * PSLOT));
    t[0] += v01.x;
    if (K > 1) t[1] += v01.y;
    if (K > 2) t[2] += __ldcg(slot + (size_t)i * PSLOT + 2);
  }
#pragma unroll
  for (int k = 0; k < K; k++) {
#pragma unroll
    for (int o = 16; o; o >>= 1) t[k] += __shfl_xor_sync(0xffffffffu, t[k], o);
    if (lane == 0) s_red[k * NW + w] = t[k];
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < NW; i++) s += s_red[threadIdx.x * NW + i];
    s_tot[threadIdx.x] = s;
  }
  __syncthreads();
}

// The solve of one system by nb CTAs, this CTA being number blk of them
// (k_pcg: the whole grid; k_pcg_groups: one group of a grouped launch).
// The shared arrays are the caller's.
template <int BS, int G, class V, class X, bool RELIABLE>
__device__ __forceinline__ void pcg_body(const PArgs& a, int nb, int blk, int init, int it_end, double* s_red,
                                         double* s_tot, int& s_abort) {
  constexpr int NG = PT / G;  // row groups per CTA
  if (threadIdx.x == 0) s_abort = 0;
  const int tid = threadIdx.x;
  const int gl = tid % G, grp = tid / G;
  const int64_t rows_per = (a.nrows + nb - 1) / nb;
  const int64_t r0 = min(a.nrows, (int64_t)blk * rows_per), r1 = min(a.nrows, r0 + rows_per);
  const int64_t e0 = r0 * BS, e1 = r1 * BS;
  X* xs = (X*)a.xs;
  X* r = (X*)a.r;
  X* z = (X*)a.z;
  X* p = (X*)a.p;
  X* q = (X*)a.q;
  const X* dinv = (const X*)a.dinv;
  const V* val = (const V*)a.val;
  double* slot0 = a.part;
  double* slot1 = a.part + (size_t)nb * PSLOT;
  double* slot2 = a.part + (size_t)2 * nb * PSLOT;
  uint32_t nbar = 0;
  PState S = *a.st;
  __syncthreads();

  if (init == 2) {
    // continuation of a stalled FP32 run in FP64: x holds the FP64
    // solution; r = b - A x, z = Dinv r, p = z (the iteration count and
    // ||b|| carry over)
    double v[2] = {0.0, 0.0};
    for (int64_t base = r0; base < r1; base += NG) {
      int64_t row = base + grp;
      const bool valid = row < r1;
      if (!valid) row = r1 - 1;
      double o[BS];
      row_dot<BS, G, double, double, double, true>(a.rowptr, a.colind, a.val64, a.x, row, gl, o);
      if (gl == 0 && valid) {
#pragma unroll
        for (int c = 0; c < BS; c++) {
          const int64_t i = row * BS + c;
          const double ri = a.b[i] - o[c];
          const X rx = (X)ri, zx = dinv[i] * rx;
          r[i] = rx;
          z[i] = zx;
          xs[i] = (X)0;
          v[0] += (double)rx * (double)zx;
          v[1] += ri * ri;
        }
      }
    }
    cta_sum<2>(v, s_red, slot2 + (size_t)blk * PSLOT);
    if (!grid_sync(a.bar, (++nbar) * nb, a.err, &s_abort)) return;
    grid_total<2>(slot2, nb, s_red, s_tot);
    // the FP64 iteration restarts from the true residual (p = z): the FP32
    // run stalled, so its direction no longer fits the true residual, and
    // continuing it made the FP64 recurrence stagnate or diverge at
    // tolerances near the attainable accuracy (measured)
    for (int64_t i = e0 + tid; i < e1; i += PT) p[i] = z[i];
    S.rz = s_tot[0];
    S.rr = s_tot[1];
    S.rmax2 = S.rr;
    S.it_upd = S.iters;
    S.max_cyc = 0;
    S.stall = 0;
    S.done = S.rr <= S.tol2;
    if (!grid_sync(a.bar, (++nbar) * nb, a.err, &s_abort)) return;
  } else if (init) {
    // r = b - A x0 (FP64 products), z = Dinv r, p = z, xs = 0; r.z, r.r, b.b
    double v[3] = {0.0, 0.0, 0.0};
    for (int64_t base = r0; base < r1; base += NG) {
      int64_t row = base + grp;
      const bool valid = row < r1;
      if (!valid) row = r1 - 1;
      double o[BS];
      if constexpr (RELIABLE) row_dot<BS, G, double, double, double, true>(a.rowptr, a.colind, a.val64, a.x, row, gl, o);
      else row_dot<BS, G, V, double, double, true>(a.rowptr, a.colind, val, a.x, row, gl, o);
      if (gl == 0 && valid) {
#pragma unroll
        for (int c = 0; c < BS; c++) {
          const int64_t i = row * BS + c;
          const double bi = a.b[i], ri = bi - o[c];
          const X rx = (X)ri, zx = dinv[i] * rx;
          r[i] = rx;
          z[i] = zx;
          p[i] = zx;
          xs[i] = (X)0;
          v[0] += (double)rx * (double)zx;
          v[1] += ri * ri;
          v[2] += bi * bi;
        }
      }
    }
    cta_sum<3>(v, s_red, slot2 + (size_t)blk * PSLOT);
    if (!grid_sync(a.bar, (++nbar) * nb, a.err, &s_abort)) return;
    grid_total<3>(slot2, nb, s_red, s_tot);
    S.rz = s_tot[0];
    S.rr = s_tot[1];
    S.bb = s_tot[2];
    S.tol2 = a.rtol2 * S.bb;
    S.rmax2 = S.rr;
    S.rzold = 0.0;
    S.iters = 0;
    S.nupd = 0;
    S.done = S.rr <= S.tol2;
  }

  while (!S.done && S.iters < it_end) {
    // P1: q = A p, p.q
    double pq;
    {
      X acc = (X)0;
      for (int64_t base = r0; base < r1; base += 2 * NG) {
        int64_t ra = base + grp, rb = base + NG + grp;
        const bool va = ra < r1, vb = rb < r1;
        if (!va) ra = r1 - 1;
        if (!vb) rb = r1 - 1;
        X oa[BS], ob[BS];
        row_dot<BS, G, V, X, X, true>(a.rowptr, a.colind, val, p, ra, gl, oa);
        row_dot<BS, G, V, X, X, true>(a.rowptr, a.colind, val, p, rb, gl, ob);
        if (gl == 0) {
#pragma unroll
          for (int c = 0; c < BS; c++) {
            if (va) {
              q[ra * BS + c] = oa[c];
              acc += oa[c] * __ldcg(p + ra * BS + c);
            }
            if (vb) {
              q[rb * BS + c] = ob[c];
              acc += ob[c] * __ldcg(p + rb * BS + c);
            }
          }
        }
      }
      double v[1] = {(double)acc};
      cta_sum<1>(v, s_red, slot0 + (size_t)blk * PSLOT);
      if (!grid_sync(a.bar, (++nbar) * nb, a.err, &s_abort)) return;
      grid_total<1>(slot0, nb, s_red, s_tot);
      pq = s_tot[0];
    }
    const X alpha = (X)(S.rz / pq);
    // P2: xs += alpha p, r -= alpha q, z = Dinv r; r.z, r.r
    double rzn, rr;
    {
      X v0 = (X)0, v1 = (X)0;
#pragma unroll 4
      for (int64_t i = e0 + tid; i < e1; i += PT) {
        const X ri = r[i] - alpha * q[i];
        const X zi = dinv[i] * ri;
        xs[i] += alpha * p[i];
        r[i] = ri;
        z[i] = zi;
        v0 += ri * zi;
        v1 += ri * ri;
      }
      double v[2] = {(double)v0, (double)v1};
      cta_sum<2>(v, s_red, slot1 + (size_t)blk * PSLOT);
      if (!grid_sync(a.bar, (++nbar) * nb, a.err, &s_abort)) return;
      grid_total<2>(slot1, nb, s_red, s_tot);
      rzn = s_tot[0];
      rr = s_tot[1];
    }
    S.iters += 1;
    double beta = rzn / S.rz;
    S.rzold = S.rz;
    S.rz = rzn;
    S.rr = rr;
    const bool stop = rr <= S.tol2 || S.iters >= a.maxit || !(rr == rr);
    if constexpr (RELIABLE) {
      // an FP32 cycle (recurrence residual down by delta) that runs past 2.5x
      // the longest earlier cycle: the FP32 iteration has lost the rate of
      // the exact iteration (eps32 * cond(A) too large); hand over to FP64
      const int cyc = S.iters - S.it_upd;
      const bool slow = sizeof(X) < sizeof(double) && (cyc > kSlowCycle || (S.max_cyc > 0 && cyc > (5 * S.max_cyc) / 2 + 16));
      if (stop || slow || rr <= a.delta2 * S.rmax2) {
        // P3: x += xs
        for (int64_t i = e0 + tid; i < e1; i += PT) {
          a.x[i] += (double)xs[i];
          xs[i] = (X)0;
        }
        if (!grid_sync(a.bar, (++nbar) * nb, a.err, &s_abort)) return;
        // P4: true residual in FP64
        double v[2] = {0.0, 0.0};
        for (int64_t base = r0; base < r1; base += NG) {
          int64_t row = base + grp;
          const bool valid = row < r1;
          if (!valid) row = r1 - 1;
          double o[BS];
          row_dot<BS, G, double, double, double, true>(a.rowptr, a.colind, a.val64, a.x, row, gl, o);
          if (gl == 0 && valid) {
#pragma unroll
            for (int c = 0; c < BS; c++) {
              const int64_t i = row * BS + c;
              const double ri = a.b[i] - o[c];
              const X rx = (X)ri, zx = dinv[i] * rx;
              r[i] = rx;
              z[i] = zx;
              v[0] += (double)rx * (double)zx;
              v[1] += ri * ri;
            }
          }
        }
        cta_sum<2>(v, s_red, slot2 + (size_t)blk * PSLOT);
        if (!grid_sync(a.bar, (++nbar) * nb, a.err, &s_abort)) return;
        grid_total<2>(slot2, nb, s_red, s_tot);
        beta = S.rzold != 0.0 ? s_tot[0] / S.rzold : 0.0;
        // the recurrence lost track of the true residual (an FP64 run past
        // its attainable accuracy, or FP32 drift): the next direction
        // restarts from the true residual instead of scaling the old one by
        // the true/recurrence mismatch
        if (s_tot[0] > (sizeof(X) == sizeof(double) ? kRestartRatio64 : kRestartRatio) * S.rz) beta = 0.0;
        const double prev = S.rmax2;
        S.rz = s_tot[0];
        S.rr = s_tot[1];
        S.rmax2 = s_tot[1];
        S.nupd += 1;
        S.done = s_tot[1] <= S.tol2 || S.iters >= a.maxit || !(s_tot[1] == s_tot[1]);
        if (sizeof(X) == sizeof(double) && !S.done) {
          // FP64: true-residual checks that do not halve ||r||, kStagnation
          // times running -- the tolerance lies below the attainable accuracy
          // (eps64 * cond(A)); the solve ends, not converged
          S.stall = s_tot[1] > 0.25 * prev ? S.stall + 1 : 0;
          if (S.stall >= kStagnation) S.done = 1;
        }
        if (sizeof(X) < sizeof(double) && !S.done) {
          // the recurrence fell by delta but the true residual did not halve:
          // the FP32 operator no longer resolves the error (eps32 * cond ~ 1)
          S.stall = s_tot[1] > a.stall_ratio * prev ? S.stall + 1 : 0;
          if (S.stall >= a.stall_count || slow) S.done = 2;
        }
        if (cyc > S.max_cyc) S.max_cyc = cyc;
        S.it_upd = S.iters;
      }
    } else {
      S.done = stop;
    }
    if (S.done) break;
    // P5: p = z + beta p
    const X bx = (X)beta;
#pragma unroll 4
    for (int64_t i = e0 + tid; i < e1; i += PT) p[i] = z[i] + bx * p[i];
    if (!grid_sync(a.bar, (++nbar) * nb, a.err, &s_abort)) return;
  }
  if (!RELIABLE && S.done) {
    for (int64_t i = e0 + tid; i < e1; i += PT) {
      a.x[i] += (double)xs[i];
      xs[i] = (X)0;
    }
  }
  if (blk == 0 && tid == 0) *a.st = S;
}

template <int BS, int G, class V, class X, bool RELIABLE>
__global__ void __launch_bounds__(PT) k_pcg(PArgs a, int init, int it_end) {
  __shared__ double s_red[3 * NW];
  __shared__ double s_tot[4];
  __shared__ int s_abort;
  pcg_body<BS, G, V, X, RELIABLE>(a, gridDim.x, blockIdx.x, init, it_end, s_red, s_tot, s_abort);
}

// Several systems in one cooperative launch: CTA c is CTA map[c].y of the
// args[map[c].x].nb CTAs that solve system map[c].x, exactly as that
// system's own launch would (its barrier, its partial slots), for `chunk`
// more iterations than its count at entry.
template <int BS, int G, class V, class X, bool RELIABLE>
__global__ void __launch_bounds__(PT) k_pcg_groups(const PArgs* __restrict__ args, const int2* __restrict__ map,
                                                   int init, int chunk) {
  __shared__ double s_red[3 * NW];
  __shared__ double s_tot[4];
  __shared__ int s_abort;
  const int2 m = map[blockIdx.x];
  const PArgs a = args[m.x];
  int it_end = a.st->iters + chunk;
  if (it_end > a.maxit || it_end < 0) it_end = a.maxit;
  pcg_body<BS, G, V, X, RELIABLE>(a, a.nb, m.y, init, it_end, s_red, s_tot, s_abort);
}

template <int BS, class V, class X>
__global__ void k_pdinv(const int64_t* rowptr, const int32_t* diag_pos, const V* val, int64_t nbrows, X* dinv) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nbrows * BS) return;
  int64_t r = t / BS;
  int c = (int)(t - r * BS);
  int64_t k = rowptr[r] + diag_pos[r];
  dinv[t] = (X)(1.0 / (double)val[k * BS * BS + c * BS + c]);
}

int lanes_for(const Matrix* A) { return row_lanes(A->nbrows > 0 ? (double)A->bnnz / (double)A->nbrows : 1.0); }

// result of one persistent run; a stalled FP32 run keeps its direction p32
// for the FP64 continuation
struct PRun {
  PState st{};
  bool stalled = false;
  float* p32 = nullptr;
};

// One system's persistent solve: its CTA count (as many as give two row
// passes per CTA, at most the co-resident CTAs of k_pcg), its buffers and
// its kernel arguments.
template <int BS, int G, class V, class X, bool REL>
struct PSolve {
  Matrix* A = nullptr;
  int nb = 0;
  X *xs = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr;
  double* part = nullptr;
  uint32_t* bar = nullptr;  // own (stand-alone) or a slot of a grouped launch's array
  int32_t* err = nullptr;
  PState* st = nullptr;
  bool own_sync = true;     // bar, err and st allocated here
  PArgs args{};
};

template <int BS, int G, class V, class X, bool REL>
static int pcg_ctas(Ctx* ctx, const Matrix* A, int* nb) {
  int per_sm = 0;
  GT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg<BS, G, V, X, REL>, PT, 0));
  if (per_sm < 1) return set_error(ctx, GT_ERR_CUDA, "persistent PCG kernel does not fit on an SM");
  constexpr int NG = PT / G;
  int64_t want = (A->nbrows + 2 * NG - 1) / (2 * NG);  // at least two row passes per CTA
  int64_t cap = (int64_t)per_sm * ctx->num_sms;
  *nb = (int)(want < cap ? (want > 0 ? want : 1) : cap);
  return GT_OK;
}

// buffers, the start state (zero, or a continuation's) and the Jacobi
// diagonal of one system; bar / err / st come from the caller when given
template <int BS, int G, class V, class X, bool REL>
static int pcg_prepare(PSolve<BS, G, V, X, REL>& P, Matrix* A, const V* val, const double* b, double* x,
                       double rtol, int maxit, double delta, const PRun* from, uint32_t* bar = nullptr,
                       int32_t* err = nullptr, PState* st = nullptr) {
  Ctx* ctx = A->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n = A->nbrows * BS;
  P.A = A;
  GT_TRY((pcg_ctas<BS, G, V, X, REL>(ctx, A, &P.nb)));
  GT_TRY(dalloc(ctx, &P.xs, n));
  GT_TRY(dalloc(ctx, &P.r, n));
  GT_TRY(dalloc(ctx, &P.z, n));
  GT_TRY(dalloc(ctx, &P.p, n));
  GT_TRY(dalloc(ctx, &P.q, n));
  GT_TRY(dalloc(ctx, &P.dinv, n));
  GT_TRY(dalloc(ctx, &P.part, (int64_t)3 * P.nb * PSLOT));
  P.own_sync = bar == nullptr;
  if (P.own_sync) {
    GT_TRY(dalloc(ctx, &P.bar, 2));
    GT_TRY(dalloc(ctx, &P.err, 2));
    GT_TRY(dalloc(ctx, (unsigned char**)&P.st, sizeof(PState)));
    GT_CUDA(ctx, cudaMemsetAsync(P.err, 0, 2 * sizeof(int32_t), s));
  } else {
    P.bar = bar;
    P.err = err;
    P.st = st;
  }
  if (from) {
    // continuation: scalars of the FP32 run (iteration count, ||b||, rzold)
    PState* h0 = reinterpret_cast<PState*>(ctx->h_dscratch);
    *h0 = from->st;
    h0->done = 0;
    GT_CUDA(ctx, cudaMemcpyAsync(P.st, h0, sizeof(PState), cudaMemcpyHostToDevice, s));
    GT_CUDA(ctx, cudaStreamSynchronize(s));
  } else {
    GT_CUDA(ctx, cudaMemsetAsync(P.st, 0, sizeof(PState), s));
  }
  GT_TRY(find_diag(A));
  const double* dval = REL ? A->val64 : (const double*)nullptr;
  if (REL || A->val64)
    k_pdinv<BS, double, X><<<GT_KC(ctx, grid_for(n, 256)), 256, 0, s>>>(A->rowptr, A->diag_pos, A->val64, A->nbrows,
                                                                         P.dinv);
  else
    k_pdinv<BS, V, X><<<GT_KC(ctx, grid_for(n, 256)), 256, 0, s>>>(A->rowptr, A->diag_pos, val, A->nbrows, P.dinv);
  GT_LAUNCH(ctx, "k_pdinv");
  PArgs& args = P.args;
  args.rowptr = A->rowptr;
  args.colind = A->colind;
  args.val = val;
  args.val64 = dval;
  args.nrows = A->nbrows;
  args.nb = P.nb;
  args.b = b;
  args.x = x;
  args.xs = P.xs;
  args.r = P.r;
  args.z = P.z;
  args.p = P.p;
  args.q = P.q;
  args.dinv = P.dinv;
  args.pcont = from ? from->p32 : nullptr;
  args.part = P.part;
  args.bar = P.bar;
  args.err = P.err;
  args.st = P.st;
  args.rtol2 = rtol * rtol;
  args.delta2 = delta * delta;
  args.maxit = maxit;
  args.stall_ratio = ctx->ir_stall_ratio;
  args.stall_count = ctx->ir_stall_count;
  return GT_OK;
}

// the outcome of a finished system (h: its final state; err: a barrier timed
// out) and the release of its buffers (a stalled FP32 run keeps p for the
// FP64 continuation)
template <int BS, int G, class V, class X, bool REL>
static int pcg_finish(PSolve<BS, G, V, X, REL>& P, const PState& h, bool err, PRun* out) {
  Ctx* ctx = P.A->ctx;
  int status = GT_OK;
  if (err) status = set_error(ctx, GT_ERR_TIMEOUT, "persistent PCG: a grid barrier timed out");
  out->st = h;
  if (status == GT_OK && h.done == 2) {
    status = PCG_STALLED;
    out->stalled = true;
    if constexpr (sizeof(X) == sizeof(float)) {
      out->p32 = reinterpret_cast<float*>(P.p);
      P.p = nullptr;
    }
  } else if (status == GT_OK && !(h.rr <= h.tol2)) {
    status = GT_ERR_NOT_CONVERGED;
  }
  dfree(ctx, P.xs);
  dfree(ctx, P.r);
  dfree(ctx, P.z);
  dfree(ctx, P.p);
  dfree(ctx, P.q);
  dfree(ctx, P.dinv);
  dfree(ctx, P.part);
  if (P.own_sync) {
    dfree(ctx, P.bar);
    dfree(ctx, P.err);
    pool_free(ctx, P.st);
  }
  return status;
}

template <int BS, int G, class V, class X, bool REL>
int run_typed(Matrix* A, const V* val, const double* b, double* x, double rtol, int maxit, double delta,
              const PRun* from, PRun* out) {
  Ctx* ctx = A->ctx;
  cudaStream_t s = ctx->stream;
  auto kern = k_pcg<BS, G, V, X, REL>;
  PSolve<BS, G, V, X, REL> P;
  GT_TRY((pcg_prepare<BS, G, V, X, REL>(P, A, val, b, x, rtol, maxit, delta, from)));
  PArgs& args = P.args;
  PState h{};
  bool err = false;
  int chunk = 32, done_iters = from ? from->st.iters : 0;
  for (int launch = 0;; launch++) {
    int init = launch == 0 ? (from ? 2 : 1) : 0;
    int it_end = done_iters + chunk;
    if (it_end > maxit || it_end < 0) it_end = maxit;
    GT_CUDA(ctx, cudaMemsetAsync(P.bar, 0, sizeof(uint32_t), s));
    void* kargs[] = {&args, &init, &it_end};
    ctx->launches++;
    GT_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)kern, dim3(P.nb), dim3(PT), kargs, 0, s));
    GT_CUDA(ctx, cudaMemcpyAsync(ctx->h_dscratch, P.st, sizeof(PState), cudaMemcpyDeviceToHost, s));
    GT_CUDA(ctx, cudaMemcpyAsync(ctx->h_scratch, P.err, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    GT_CUDA(ctx, cudaStreamSynchronize(s));
    memcpy(&h, ctx->h_dscratch, sizeof(PState));
    int32_t e = 0;
    memcpy(&e, ctx->h_scratch, sizeof(int32_t));
    if (e) {
      err = true;
      break;
    }
    done_iters = h.iters;
    if (h.done || h.iters >= maxit) break;
    if (chunk < 2048) chunk *= 2;
  }
  return pcg_finish<BS, G, V, X, REL>(P, h, err, out);
}

// Grouped persistent solves: systems of one block size and lane count, each
// on the CTAs its stand-alone solve would use (so its partition, its
// reductions and its result are bitwise that solve's), packed in order into
// cooperative launches whose CTAs are co-resident; every system waits only
// on its own bounded barrier.  All systems of one call start alike (froms
// all null, or all continuations).  A system larger than one launch holds
// is solved stand-alone.
template <int BS, int G, class V, class X, bool REL>
static int run_groups_typed(Ctx* ctx, const std::vector<Matrix*>& As, const std::vector<const V*>& vals,
                            const std::vector<const double*>& bs, const std::vector<double*>& xs, double rtol,
                            int maxit, double delta, const std::vector<const PRun*>& froms, std::vector<PRun>& outs,
                            std::vector<int>& status) {
  cudaStream_t s = ctx->stream;
  const int n = (int)As.size();
  auto kern = k_pcg_groups<BS, G, V, X, REL>;
  int per_sm = 0;
  GT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PT, 0));
  const int64_t cap = (int64_t)(per_sm > 0 ? per_sm : 0) * ctx->num_sms;
  std::vector<int> nbs(n);
  for (int i = 0; i < n; i++) GT_TRY((pcg_ctas<BS, G, V, X, REL>(ctx, As[i], &nbs[i])));
  int i0 = 0;
  while (i0 < n) {
    int i1 = i0;
    int64_t tot = 0;
    while (i1 < n && tot + nbs[i1] <= cap) tot += nbs[i1++];
    if (i1 == i0) {
      status[i0] = run_typed<BS, G, V, X, REL>(As[i0], vals[i0], bs[i0], xs[i0], rtol, maxit, delta, froms[i0],
                                               &outs[i0]);
      i0++;
      continue;
    }
    const int m = i1 - i0;
    uint32_t* bars = nullptr;
    int32_t* errs = nullptr;
    PState* sts = nullptr;
    PArgs* dargs = nullptr;
    int2* dmap = nullptr;
    std::vector<PSolve<BS, G, V, X, REL>> P(m);
    int prepared = 0;
    std::vector<PState> h(m);
    bool err = false;
    // one wave; every exit below goes through the release of its blocks
    auto wave = [&]() -> int {
      GT_TRY(dalloc(ctx, &bars, 2 * (int64_t)m));
      GT_TRY(dalloc(ctx, &errs, 2 * (int64_t)m));
      GT_TRY(dalloc(ctx, (unsigned char**)&sts, (int64_t)sizeof(PState) * m));
      GT_TRY(dalloc(ctx, (unsigned char**)&dargs, (int64_t)sizeof(PArgs) * m));
      GT_TRY(dalloc(ctx, (unsigned char**)&dmap, (int64_t)sizeof(int2) * tot));
      GT_CUDA(ctx, cudaMemsetAsync(errs, 0, sizeof(int32_t) * 2 * m, s));
      std::vector<PArgs> hargs(m);
      std::vector<int2> hmap;
      hmap.reserve(tot);
      for (int k = 0; k < m; k++, prepared++) {
        const int i = i0 + k;
        GT_TRY((pcg_prepare<BS, G, V, X, REL>(P[k], As[i], vals[i], bs[i], xs[i], rtol, maxit, delta, froms[i],
                                              bars + 2 * k, errs + 2 * k, sts + k)));
        hargs[k] = P[k].args;
        for (int j = 0; j < P[k].nb; j++) hmap.push_back(make_int2(k, j));
      }
      GT_TRY(copy_in(ctx, (unsigned char*)dargs, (const unsigned char*)hargs.data(), (int64_t)sizeof(PArgs) * m));
      GT_TRY(copy_in(ctx, (unsigned char*)dmap, (const unsigned char*)hmap.data(), (int64_t)sizeof(int2) * tot));
      std::vector<int32_t> e(2 * m, 0);
      int chunk = 32;
      for (int launch = 0;; launch++) {
        int init = launch == 0 ? (froms[i0] ? 2 : 1) : 0;
        GT_CUDA(ctx, cudaMemsetAsync(bars, 0, sizeof(uint32_t) * 2 * m, s));
        void* kargs[] = {&dargs, &dmap, &init, &chunk};
        ctx->launches++;
        GT_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)kern, dim3((unsigned)tot), dim3(PT), kargs, 0, s));
        GT_CUDA(ctx, cudaMemcpyAsync(h.data(), sts, sizeof(PState) * m, cudaMemcpyDeviceToHost, s));
        GT_CUDA(ctx, cudaMemcpyAsync(e.data(), errs, sizeof(int32_t) * 2 * m, cudaMemcpyDeviceToHost, s));
        GT_CUDA(ctx, cudaStreamSynchronize(s));
        bool all = true;
        for (int k = 0; k < m; k++) {
          err |= e[2 * k] != 0;
          all &= h[k].done != 0 || h[k].iters >= maxit;
        }
        if (err || all) break;
        if (chunk < 2048) chunk *= 2;
      }
      return GT_OK;
    };
    const int ws = wave();
    if (ws != GT_OK) cudaStreamSynchronize(s);  // nothing of the wave may be reused before the stream drains
    for (int k = 0; k < prepared; k++) {
      const int st = pcg_finish<BS, G, V, X, REL>(P[k], h[k], err, &outs[i0 + k]);
      status[i0 + k] = ws == GT_OK ? st : ws;
    }
    dfree(ctx, bars);
    dfree(ctx, errs);
    pool_free(ctx, sts);
    pool_free(ctx, dargs);
    pool_free(ctx, dmap);
    if (ws != GT_OK) return ws;
    i0 = i1;
  }
  return GT_OK;
}

template <class V, class X, bool REL>
static int run_groups_dispatch(Ctx* ctx, int bs, int G, const std::vector<Matrix*>& As,
                               const std::vector<const V*>& vals, const std::vector<const double*>& b,
                               const std::vector<double*>& x, double rtol, int maxit, double delta,
                               const std::vector<const PRun*>& froms, std::vector<PRun>& outs,
                               std::vector<int>& status) {
#define GT_PCGG_CASE(BS_, G_)                                                                                  \
  if (bs == BS_ && G == G_)                                                                                    \
    return run_groups_typed<BS_, G_, V, X, REL>(ctx, As, vals, b, x, rtol, maxit, delta, froms, outs, status);
  GT_PCGG_CASE(1, 1) GT_PCGG_CASE(1, 2) GT_PCGG_CASE(1, 4) GT_PCGG_CASE(1, 8)
  GT_PCGG_CASE(3, 1) GT_PCGG_CASE(3, 2) GT_PCGG_CASE(3, 4) GT_PCGG_CASE(3, 8)
#undef GT_PCGG_CASE
  return set_error(ctx, GT_ERR_UNSUPPORTED, "grouped persistent PCG: unsupported block size");
}

template <class V, class X, bool REL>
int run_dispatch(Matrix* A, const V* val, const double* b, double* x, double rtol, int maxit, double delta,
                 const PRun* from, PRun* out) {
  const int G = lanes_for(A);
#define GT_PCG_CASE(BS_, G_)                                                                                   \
  if (A->bs == BS_ && G == G_) return run_typed<BS_, G_, V, X, REL>(A, val, b, x, rtol, maxit, delta, from, out);
  GT_PCG_CASE(1, 1) GT_PCG_CASE(1, 2) GT_PCG_CASE(1, 4) GT_PCG_CASE(1, 8)
  GT_PCG_CASE(2, 1) GT_PCG_CASE(2, 2) GT_PCG_CASE(2, 4) GT_PCG_CASE(2, 8)
  GT_PCG_CASE(3, 1) GT_PCG_CASE(3, 2) GT_PCG_CASE(3, 4) GT_PCG_CASE(3, 8)
#undef GT_PCG_CASE
  return set_error(A->ctx, GT_ERR_UNSUPPORTED, "persistent PCG: unsupported block size");
}

// The solver's grid barrier run alone: `ctas` co-resident CTAs wait for
// ctas + missing arrivals.  With missing > 0 the barrier can never complete,
// so each CTA gives up after timeout_ns and sets the error word.
__global__ void __launch_bounds__(PT) k_barrier_probe(uint32_t* bar, uint32_t target, int32_t* err,
                                                      uint64_t timeout_ns) {
  __shared__ int s_abort;
  if (threadIdx.x == 0) s_abort = 0;
  grid_sync(bar, target, err, &s_abort, timeout_ns);
}

}  // namespace

int barrier_probe(Ctx* ctx, int ctas, int missing, int64_t timeout_ns) {
  if (ctas < 1 || missing < 0 || timeout_ns <= 0 || timeout_ns > 2000000000ll)
    return set_error(ctx, GT_ERR_INVALID, "barrier probe: 1 <= ctas, 0 <= missing, 0 < timeout <= 2 s");
  int dev = 0, nsm = 0, per_sm = 0;
  GT_CUDA(ctx, cudaGetDevice(&dev));
  GT_CUDA(ctx, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  GT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_barrier_probe, PT, 0));
  if ((int64_t)ctas > (int64_t)nsm * per_sm) return set_error(ctx, GT_ERR_INVALID, "barrier probe: more CTAs than fit");
  cudaStream_t s = ctx->stream;
  uint32_t* bar = nullptr;
  int32_t* err = nullptr;
  GT_TRY(dalloc(ctx, &bar, 2));
  GT_TRY(dalloc(ctx, &err, 2));
  GT_CUDA(ctx, cudaMemsetAsync(bar, 0, 2 * sizeof(uint32_t), s));
  GT_CUDA(ctx, cudaMemsetAsync(err, 0, 2 * sizeof(int32_t), s));
  uint32_t target = (uint32_t)(ctas + missing);
  uint64_t tns = (uint64_t)timeout_ns;
  void* kargs[] = {&bar, &target, &err, &tns};
  ctx->launches++;
  GT_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)k_barrier_probe, dim3(ctas), dim3(PT), kargs, 0, s));
  GT_CUDA(ctx, cudaMemcpyAsync(ctx->h_scratch, err, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GT_CUDA(ctx, cudaStreamSynchronize(s));
  int32_t e = 0;
  memcpy(&e, ctx->h_scratch, sizeof(int32_t));
  dfree(ctx, bar);
  dfree(ctx, err);
  return e ? set_error(ctx, GT_ERR_TIMEOUT, "barrier probe: the grid barrier timed out") : GT_OK;
}

// pcg_persistent for several systems of ctx (FP64 or FP32 with reliable
// updates), grouped into shared cooperative launches by block size and
// lane count; x: start values; per-system infos and statuses.  Each system's
// result is bitwise that of pcg_persistent on it alone.
int pcg_persistent_groups(Ctx* ctx, const std::vector<Matrix*>& As, int mode, const std::vector<const double*>& b,
                          const std::vector<double*>& x, double rtol, int maxit, std::vector<gt_solve_info>& infos,
                          std::vector<int>& status) {
  const int n = (int)As.size();
  infos.assign(n, gt_solve_info{});
  status.assign(n, GT_OK);
  if (mode != GT_SOLVE_FP64 && mode != GT_SOLVE_IR)
    return set_error(ctx, GT_ERR_INVALID, "grouped persistent PCG: FP64 or mixed mode");
  std::vector<PRun> runs(n);
  for (int bs : {1, 3})
    for (int g : {1, 2, 4, 8}) {
      std::vector<int> ids;
      for (int i = 0; i < n; i++)
        if (As[i]->bs == bs && lanes_for(As[i]) == g) ids.push_back(i);
      if (ids.empty()) continue;
      std::vector<Matrix*> A;
      std::vector<const double*> bb;
      std::vector<double*> xx;
      std::vector<const PRun*> none(ids.size(), nullptr);
      std::vector<PRun> out(ids.size());
      std::vector<int> st(ids.size(), GT_OK);
      for (int i : ids) {
        A.push_back(As[i]);
        bb.push_back(b[i]);
        xx.push_back(x[i]);
      }
      if (mode == GT_SOLVE_FP64) {
        std::vector<const double*> v;
        for (Matrix* M : A) v.push_back(M->val64);
        GT_TRY((run_groups_dispatch<double, double, true>(ctx, bs, g, A, v, bb, xx, rtol, maxit, 0.0, none, out, st)));
        for (size_t k = 0; k < ids.size(); k++) infos[ids[k]].fp64_iterations = out[k].st.iters;
      } else {
        std::vector<const float*> v;
        for (Matrix* M : A) v.push_back(M->val32);
        GT_TRY((run_groups_dispatch<float, float, true>(ctx, bs, g, A, v, bb, xx, rtol, maxit, ctx->ir_delta, none,
                                                        out, st)));
        // stalled FP32 runs go on in FP64 from their FP64 solutions, as alone
        std::vector<size_t> sk;
        for (size_t k = 0; k < ids.size(); k++)
          if (st[k] == PCG_STALLED) sk.push_back(k);
        if (!sk.empty()) {
          std::vector<Matrix*> A2;
          std::vector<const double*> v2, b2;
          std::vector<double*> x2;
          std::vector<const PRun*> f2;
          for (size_t k : sk) {
            A2.push_back(A[k]);
            v2.push_back(A[k]->val64);
            b2.push_back(bb[k]);
            x2.push_back(xx[k]);
            f2.push_back(&out[k]);
          }
          std::vector<PRun> o2(sk.size());
          std::vector<int> s2(sk.size(), GT_OK);
          int e = run_groups_dispatch<double, double, true>(ctx, bs, g, A2, v2, b2, x2, rtol, maxit, 0.0, f2, o2, s2);
          for (size_t k : sk)
            if (out[k].p32) pool_free(ctx, out[k].p32);
          GT_TRY(e);
          for (size_t j = 0; j < sk.size(); j++) {
            infos[ids[sk[j]]].fp64_iterations = o2[j].st.iters - out[sk[j]].st.iters;
            out[sk[j]] = o2[j];
            st[sk[j]] = s2[j];
          }
        }
      }
      for (size_t k = 0; k < ids.size(); k++) {
        gt_solve_info& inf = infos[ids[k]];
        inf.iterations = out[k].st.iters;
        inf.outer_iterations = out[k].st.nupd;
        inf.rel_residual = out[k].st.bb > 0 ? sqrt(out[k].st.rr / out[k].st.bb) : 0.0;
        status[ids[k]] = st[k];
      }
    }
  return GT_OK;
}

int pcg_persistent(Matrix* A, int mode, const double* b, double* x, double rtol, int maxit, int32_t* iters,
                   int32_t* nupd, int32_t* iters64, double* relres) {
  PRun run;
  int s;
  *iters64 = 0;
  if (mode == GT_SOLVE_FP64) {
    s = run_dispatch<double, double, true>(A, A->val64, b, x, rtol, maxit, 0.0, nullptr, &run);
    *iters64 = run.st.iters;
  } else if (mode == GT_SOLVE_IR) {
    s = run_dispatch<float, float, true>(A, A->val32, b, x, rtol, maxit, A->ctx->ir_delta, nullptr, &run);
    if (s == PCG_STALLED) {
      // the FP32 iteration stalled or lost its rate (eps32 * cond(A) too
      // large): the same Krylov iteration goes on in FP64 from the current
      // FP64 solution and the FP32 direction
      PRun r32 = run;
      PRun r64;
      s = run_dispatch<double, double, true>(A, A->val64, b, x, rtol, maxit, 0.0, &r32, &r64);
      if (r32.p32) pool_free(A->ctx, r32.p32);
      *iters64 = r64.st.iters - r32.st.iters;
      run = r64;
    }
  } else {
    s = run_dispatch<float, float, false>(A, A->val32, b, x, rtol, maxit, 0.0, nullptr, &run);
  }
  *iters = run.st.iters;
  *nupd = run.st.nupd;
  *relres = run.st.bb > 0 ? sqrt(run.st.rr / run.st.bb) : 0.0;
  return s;
}

}  // namespace gt
