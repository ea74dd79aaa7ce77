// gt_batch.cu -- many independent solves of uneven size in few launches.
//
// A batch holds n assembled matrices of block size 1 (scalar problems) or
// 3 (3-D linear elasticity).  Instances are split by size (scalar rows):
//
//  * small instances (rows <= kSmallRows) are solved by ONE persistent
//    launch: each CTA takes the next instance from a queue (largest first)
//    and runs its whole Jacobi-PCG alone -- SpMV with G lanes per row, CTA
//    reductions through shared memory, no inter-CTA synchronisation -- then
//    takes the next one, so the device stays full however uneven the sizes;
//  * medium instances (up to the persistent solver's 262,144 rows, matrices
//    of the batch's own context, FP64 or mixed mode) share cooperative
//    launches of the persistent solver: each one on the CTAs its own solve
//    would use, with its own bounded barrier, so many run at once;
//  * large instances, which fill the device by themselves, run one after
//    the other through the single-system solver of gt_solve.cu.
//
// Either way an instance's arithmetic and summation order depend only on
// the instance (one CTA in a fixed order, or the grid layout of the
// instance's own solve), so its result is bitwise the same alone and in any
// mix.  The precision modes match gt_solve: FP64 CG, FP32 CG with FP64
// reliable updates (an FP32 run that stalls or loses its rate continues in
// FP64), and FP32 CG.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gt_internal.cuh"
#include "gt_rowdot.cuh"

namespace gt {

constexpr int BT = 256;                 // threads per CTA of the batched kernel
constexpr int BNW = BT / 32;
constexpr int64_t kSmallRows = 32768;   // instances up to this size run one per CTA

struct BInst {
  const int64_t* rowptr;
  const int32_t* colind;
  const double* v64;
  const float* v32;
  const int32_t* diag;  // position of the diagonal block in each block row
  int64_t nrows;        // block rows
  int64_t off;          // offset of the instance in the concatenated vectors (scalar entries)
  int32_t bs, pad;
};

// per-instance outcome of the batched kernel
struct BRes {
  double rr, bb;        // final ||r||^2 (true residual with reliable updates) and ||b||^2
  int32_t iters, nupd;
  int32_t status;       // 0 converged, 1 maxit / breakdown, 2 FP32 stalled (continue in FP64)
  int32_t pad;
};

struct BatchImpl {
  Ctx* ctx = nullptr;
  int n = 0;
  int G = 0;  // lanes per row of the one-CTA solves; 0: each instance's own (row_lanes of its mean row)
  int64_t ntot = 0;
  std::vector<Matrix*> mats;
  std::vector<BInst> h_inst;
  BInst* d_inst = nullptr;
  int64_t small_rows = kSmallRows;  // scalar rows up to which an instance runs on one CTA
  std::vector<int> small, large;   // instance ids by class (small: largest first)
};

// the one-CTA tier: instances up to B->small_rows scalar rows, largest first
static void classify(BatchImpl* B) {
  B->small.clear();
  B->large.clear();
  for (int i = 0; i < B->n; i++) {
    if (B->h_inst[i].nrows * B->h_inst[i].bs <= B->small_rows) B->small.push_back(i);
    else B->large.push_back(i);
  }
  std::stable_sort(B->small.begin(), B->small.end(), [&](int a, int c) {
    return B->h_inst[a].nrows * B->h_inst[a].bs > B->h_inst[c].nrows * B->h_inst[c].bs;
  });
}

// CTA sum of K values, identical in every thread (fixed order); sr is one of
// two alternating shared buffers of K * BNW doubles
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* sr) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double t = v[k];
#pragma unroll
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) sr[k * BNW + w] = t;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; k++) {
    double t = 0.0;
#pragma unroll
    for (int i = 0; i < BNW; i++) t += sr[k * BNW + i];
    v[k] = t;
  }
}

template <class V>
__device__ __forceinline__ const V* inst_vals(const BInst& in) {
  if constexpr (sizeof(V) == 8) return (const V*)in.v64;
  else return (const V*)in.v32;
}

// One CTA per instance, instances from a queue.  BS: block size of the
// instances of the launch (G lanes per block row); V: values of the
// iteration, X: vector type; REL: FP64 reliable updates (needs v64).
// from_x: start from the given x (else x = 0).  Jacobi on the scalar
// diagonal, as the single-system solver.
template <int BS, int G, class V, class X, bool REL>
__global__ void __launch_bounds__(BT) k_bpcg(const BInst* __restrict__ insts, const int32_t* __restrict__ queue,
                                             int nq, int32_t* head, const double* __restrict__ b, double* x, X* xs,
                                             X* r, X* z, X* p, X* q, X* dinv, BRes* res, double rtol2, double delta2,
                                             int maxit, int from_x, double stall_ratio, int stall_count) {
  __shared__ double s_red[2][3 * BNW];
  __shared__ int s_k;
  constexpr int NG = BT / G;
  const int tid = threadIdx.x, gl = tid % G, grp = tid / G;
  int buf = 0;
  while (true) {
    if (tid == 0) s_k = atomicAdd(head, 1);
    __syncthreads();
    const int k = s_k;
    __syncthreads();
    if (k >= nq) return;
    const int ii = queue[k];
    const BInst in = insts[ii];
    const int64_t nb = in.nrows, n = nb * BS, off = in.off;
    const V* val = inst_vals<V>(in);
    const double* bi = b + off;
    double* xi = x + off;
    X *xsi = xs + off, *ri = r + off, *zi = z + off, *pi = p + off, *qi = q + off, *di = dinv + off;
    for (int64_t i = tid; i < n; i += BT) {
      const int64_t br = i / BS;
      const int c = (int)(i - br * BS);
      const int64_t pos = (in.rowptr[br] + in.diag[br]) * BS * BS + c * BS + c;
      const double d = in.v64 ? in.v64[pos] : (double)in.v32[pos];
      di[i] = (X)(1.0 / d);
      if (!from_x) xi[i] = 0.0;
    }
    __syncthreads();
    // r = b - A x, z = Dinv r, p = z, xs = 0
    double rz, rr, bb;
    {
      double v[3] = {0.0, 0.0, 0.0};
      for (int64_t base = 0; base < nb; base += NG) {
        int64_t row = base + grp;
        const bool valid = row < nb;
        if (!valid) row = nb - 1;
        double o[BS];
        if constexpr (REL) row_dot<BS, G, double, double, double, false>(in.rowptr, in.colind, in.v64, xi, row, gl, o);
        else row_dot<BS, G, V, double, double, false>(in.rowptr, in.colind, val, xi, row, gl, o);
        if (gl == 0 && valid) {
#pragma unroll
          for (int c = 0; c < BS; c++) {
            const int64_t i = row * BS + c;
            const double bv = bi[i], rv = bv - o[c];
            const X rx = (X)rv, zx = di[i] * rx;
            ri[i] = rx;
            zi[i] = zx;
            pi[i] = zx;
            xsi[i] = (X)0;
            v[0] += (double)rx * (double)zx;
            v[1] += rv * rv;
            v[2] += bv * bv;
          }
        }
      }
      block_sum<3>(v, s_red[buf]);
      buf ^= 1;
      rz = v[0];
      rr = v[1];
      bb = v[2];
    }
    const double tol2 = rtol2 * bb;
    double rmax2 = rr, rzold = 0.0;
    int iters = 0, nupd = 0, status = 0, it_upd = 0, max_cyc = 0, stall = 0;
    bool done = rr <= tol2;
    while (!done) {
      // q = A p, p.q
      double pq;
      {
        X acc = (X)0;
        for (int64_t base = 0; base < nb; base += 2 * NG) {
          int64_t ra = base + grp, rb = base + NG + grp;
          const bool va = ra < nb, vb = rb < nb;
          if (!va) ra = nb - 1;
          if (!vb) rb = nb - 1;
          X oa[BS], ob[BS];
          row_dot<BS, G, V, X, X, false>(in.rowptr, in.colind, val, pi, ra, gl, oa);
          row_dot<BS, G, V, X, X, false>(in.rowptr, in.colind, val, pi, rb, gl, ob);
          if (gl == 0) {
            if (va)
#pragma unroll
              for (int c = 0; c < BS; c++) {
                qi[ra * BS + c] = oa[c];
                acc += oa[c] * pi[ra * BS + c];
              }
            if (vb)
#pragma unroll
              for (int c = 0; c < BS; c++) {
                qi[rb * BS + c] = ob[c];
                acc += ob[c] * pi[rb * BS + c];
              }
          }
        }
        double v[1] = {(double)acc};
        block_sum<1>(v, s_red[buf]);
        buf ^= 1;
        pq = v[0];
      }
      const X alpha = (X)(rz / pq);
      double rzn;
      {
        X v0 = (X)0, v1 = (X)0;
        for (int64_t i = tid; i < n; i += BT) {
          const X rv = ri[i] - alpha * qi[i];
          const X zv = di[i] * rv;
          xsi[i] += alpha * pi[i];
          ri[i] = rv;
          zi[i] = zv;
          v0 += rv * zv;
          v1 += rv * rv;
        }
        double v[2] = {(double)v0, (double)v1};
        block_sum<2>(v, s_red[buf]);
        buf ^= 1;
        rzn = v[0];
        rr = v[1];
      }
      iters++;
      double beta = rzn / rz;
      rzold = rz;
      rz = rzn;
      const bool stop = rr <= tol2 || iters >= maxit || !(rr == rr);
      if constexpr (REL) {
        const int cyc = iters - it_upd;
        const bool slow = sizeof(X) < sizeof(double) && (cyc > kSlowCycle || (max_cyc > 0 && cyc > (5 * max_cyc) / 2 + 16));
        if (stop || slow || rr <= delta2 * rmax2) {
          for (int64_t i = tid; i < n; i += BT) {
            xi[i] += (double)xsi[i];
            xsi[i] = (X)0;
          }
          __syncthreads();
          double v[2] = {0.0, 0.0};
          for (int64_t base = 0; base < nb; base += NG) {
            int64_t row = base + grp;
            const bool valid = row < nb;
            if (!valid) row = nb - 1;
            double o[BS];
            row_dot<BS, G, double, double, double, false>(in.rowptr, in.colind, in.v64, xi, row, gl, o);
            if (gl == 0 && valid) {
#pragma unroll
              for (int c = 0; c < BS; c++) {
                const int64_t i = row * BS + c;
                const double rv = bi[i] - o[c];
                const X rx = (X)rv, zx = di[i] * rx;
                ri[i] = rx;
                zi[i] = zx;
                v[0] += (double)rx * (double)zx;
                v[1] += rv * rv;
              }
            }
          }
          block_sum<2>(v, s_red[buf]);
          buf ^= 1;
          beta = rzold != 0.0 ? v[0] / rzold : 0.0;
          // the recurrence lost track of the true residual: restart the directions
          if (v[0] > (sizeof(X) == sizeof(double) ? kRestartRatio64 : kRestartRatio) * rz) beta = 0.0;
          const double prev = rmax2;
          rz = v[0];
          rr = v[1];
          rmax2 = v[1];
          nupd++;
          done = rr <= tol2 || iters >= maxit || !(rr == rr);
          if (sizeof(X) == sizeof(double) && !done) {
            // FP64: checks that do not halve ||r||, kStagnation times running:
            // the tolerance lies below the attainable accuracy
            stall = rr > 0.25 * prev ? stall + 1 : 0;
            if (stall >= kStagnation) done = true;
          }
          if (sizeof(X) < sizeof(double) && !done) {
            stall = rr > stall_ratio * prev ? stall + 1 : 0;
            if (stall >= stall_count || slow) {
              done = true;
              status = 2;
            }
          }
          if (cyc > max_cyc) max_cyc = cyc;
          it_upd = iters;
        }
      } else {
        done = stop;
      }
      if (done) break;
      const X bx = (X)beta;
      for (int64_t i = tid; i < n; i += BT) pi[i] = zi[i] + bx * pi[i];
      __syncthreads();
    }
    if (!REL) {
      for (int64_t i = tid; i < n; i += BT) {
        xi[i] += (double)xsi[i];
        xsi[i] = (X)0;
      }
    }
    if (tid == 0) {
      BRes o{};
      o.rr = rr;
      o.bb = bb;
      o.iters = iters;
      o.nupd = nupd;
      o.status = status == 2 ? 2 : (rr <= tol2 ? 0 : 1);
      res[ii] = o;
    }
    __syncthreads();
  }
}

}  // namespace gt

struct gt_batch : gt::BatchImpl {};

namespace gt {

template <class V, class X, bool REL>
static int launch_small_g(gt_batch* B, int bs, int G, const std::vector<int>& ids, const double* b, double* x, double rtol,
                          int maxit, double delta, int from_x, std::vector<BRes>& hres) {
  Ctx* ctx = B->ctx;
  cudaStream_t s = ctx->stream;
  if (ids.empty()) return GT_OK;
  const int64_t n = B->ntot;
  X *xs = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr;
  int32_t *queue = nullptr, *head = nullptr;
  BRes* res = nullptr;
  GT_TRY(dalloc(ctx, &xs, n));
  GT_TRY(dalloc(ctx, &r, n));
  GT_TRY(dalloc(ctx, &z, n));
  GT_TRY(dalloc(ctx, &p, n));
  GT_TRY(dalloc(ctx, &q, n));
  GT_TRY(dalloc(ctx, &dinv, n));
  GT_TRY(dalloc(ctx, &queue, (int64_t)ids.size()));
  GT_TRY(dalloc(ctx, &head, 1));
  GT_TRY(dalloc(ctx, (unsigned char**)&res, (int64_t)sizeof(BRes) * B->n));
  GT_TRY(copy_in(ctx, queue, ids.data(), (int64_t)ids.size()));
  GT_CUDA(ctx, cudaMemsetAsync(head, 0, sizeof(int32_t), s));
  auto launch = [&](auto kern) -> int {
    int per_sm = 0;
    GT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BT, 0));
    int64_t cap = (int64_t)std::max(per_sm, 1) * ctx->num_sms;
    int grid = (int)std::min<int64_t>(cap, (int64_t)ids.size());
    kern<<<GT_KC(ctx, grid), BT, 0, s>>>(B->d_inst, queue, (int)ids.size(), head, b, x, xs, r, z, p, q, dinv, res,
                                         rtol * rtol, delta * delta, maxit, from_x, ctx->ir_stall_ratio,
                                         ctx->ir_stall_count);
    GT_LAUNCH(ctx, "k_bpcg");
    return GT_OK;
  };
  int st;
  if (bs == 3) {
    // block rows of 3-D elasticity: 2 or 4 lanes (inst_lanes)
    st = G == 2 ? launch(k_bpcg<3, 2, V, X, REL>) : launch(k_bpcg<3, 4, V, X, REL>);
  } else {
    switch (G) {
      case 1: st = launch(k_bpcg<1, 1, V, X, REL>); break;
      case 2: st = launch(k_bpcg<1, 2, V, X, REL>); break;
      case 8: st = launch(k_bpcg<1, 8, V, X, REL>); break;
      default: st = launch(k_bpcg<1, 4, V, X, REL>); break;
    }
  }
  if (st == GT_OK) {
    std::vector<BRes> all(B->n);
    GT_CUDA(ctx, cudaMemcpyAsync(all.data(), res, sizeof(BRes) * B->n, cudaMemcpyDeviceToHost, s));
    GT_CUDA(ctx, cudaStreamSynchronize(s));
    for (int i : ids) hres[i] = all[i];
  }
  dfree(ctx, xs);
  dfree(ctx, r);
  dfree(ctx, z);
  dfree(ctx, p);
  dfree(ctx, q);
  dfree(ctx, dinv);
  dfree(ctx, queue);
  dfree(ctx, head);
  pool_free(ctx, res);
  return st;
}

// lanes of instance i in the one-CTA solves: fixed by set_lanes, else from
// the instance's own mean row length (so the result depends on nothing
// else); block rows of 3 take 2 or 4
static int inst_lanes(const gt_batch* B, int i) {
  const Matrix* A = B->mats[i];
  int g = B->G ? B->G : row_lanes(A->nbrows > 0 ? (double)A->bnnz / (double)A->nbrows : 1.0);
  if (A->bs == 3) g = g <= 2 ? 2 : 4;
  return g;
}

// one launch per block size and lane count (instances keep their
// largest-first order)
template <class V, class X, bool REL>
static int launch_small(gt_batch* B, const std::vector<int>& ids, const double* b, double* x, double rtol, int maxit,
                        double delta, int from_x, std::vector<BRes>& hres) {
  for (int bs : {1, 3})
    for (int g : {1, 2, 4, 8}) {
      std::vector<int> sub;
      for (int i : ids)
        if (B->mats[i]->bs == bs && inst_lanes(B, i) == g) sub.push_back(i);
      if (!sub.empty()) GT_TRY((launch_small_g<V, X, REL>(B, bs, g, sub, b, x, rtol, maxit, delta, from_x, hres)));
    }
  return GT_OK;
}

static int batch_solve(gt_batch* B, const double* b, double* x, double rtol, int maxit, int mode, gt_solve_info* infos) {
  Ctx* ctx = B->ctx;
  const int ni = B->n;
  for (auto* A : B->mats) {
    if ((mode == GT_SOLVE_FP64 && !A->val64) || (mode == GT_SOLVE_FP32 && !A->val32))
      return set_error(ctx, GT_ERR_INVALID, "batch solve: matrices lack the values of this mode");
    if (mode == GT_SOLVE_IR && (!A->val64 || !A->val32))
      return set_error(ctx, GT_ERR_INVALID, "batch IR solve needs GT_MIXED matrices");
  }
  if (mode != GT_SOLVE_FP64 && mode != GT_SOLVE_FP32 && mode != GT_SOLVE_IR)
    return set_error(ctx, GT_ERR_INVALID, "unknown solve mode");
  std::vector<gt_solve_info> info(ni);
  std::vector<BRes> hres(ni);
  int status = GT_OK;
  // small instances: one persistent launch
  if (mode == GT_SOLVE_FP64) {
    GT_TRY((launch_small<double, double, true>(B, B->small, b, x, rtol, maxit, 0.0, 0, hres)));
  } else if (mode == GT_SOLVE_FP32) {
    GT_TRY((launch_small<float, float, false>(B, B->small, b, x, rtol, maxit, 0.0, 0, hres)));
  } else {
    GT_TRY((launch_small<float, float, true>(B, B->small, b, x, rtol, maxit, ctx->ir_delta, 0, hres)));
    std::vector<int> stalled;
    for (int i : B->small)
      if (hres[i].status == 2) stalled.push_back(i);
    if (!stalled.empty()) {
      // FP32 stalled (eps32 * cond ~ 1): these instances go on in FP64 from
      // their current FP64 solution
      std::vector<BRes> h64(ni);
      GT_TRY((launch_small<double, double, true>(B, stalled, b, x, rtol, maxit, 0.0, 1, h64)));
      for (int i : stalled) {
        info[i].fp64_iterations = h64[i].iters;
        h64[i].iters += hres[i].iters;
        h64[i].nupd += hres[i].nupd;
        hres[i] = h64[i];
      }
    }
  }
  for (int i : B->small) {
    info[i].iterations = hres[i].iters;
    info[i].outer_iterations = mode == GT_SOLVE_FP32 ? 0 : hres[i].nupd;
    info[i].rel_residual = hres[i].bb > 0 ? sqrt(hres[i].rr / hres[i].bb) : 0.0;
    if (mode == GT_SOLVE_FP64) info[i].fp64_iterations = hres[i].iters;
    if (hres[i].status != 0) status = GT_ERR_NOT_CONVERGED;
  }
  mark(ctx, "batch_small");
  // medium instances of this context: grouped persistent launches
  std::vector<int> rest;
  {
    std::vector<int> grouped;
    for (int i : B->large) {
      Matrix* A = B->mats[i];
      if ((mode == GT_SOLVE_FP64 || mode == GT_SOLVE_IR) && A->ctx == ctx && A->nbrows * A->bs <= kPersistentMaxRows)
        grouped.push_back(i);
      else
        rest.push_back(i);
    }
    if (!grouped.empty()) {
      std::vector<Matrix*> As;
      std::vector<const double*> bs;
      std::vector<double*> xs;
      for (int i : grouped) {
        const int64_t off = B->h_inst[i].off;
        As.push_back(B->mats[i]);
        bs.push_back(b + off);
        xs.push_back(x + off);
        GT_CUDA(ctx, cudaMemsetAsync(x + off, 0, sizeof(double) * B->mats[i]->nbrows * B->mats[i]->bs, ctx->stream));
      }
      std::vector<gt_solve_info> ginf;
      std::vector<int> gst;
      GT_TRY(pcg_persistent_groups(ctx, As, mode, bs, xs, rtol, maxit, ginf, gst));
      for (size_t k = 0; k < grouped.size(); k++) {
        info[grouped[k]] = ginf[k];
        if (gst[k] != GT_OK && gst[k] != GT_ERR_NOT_CONVERGED) return gst[k];
        if (gst[k] == GT_ERR_NOT_CONVERGED) status = gst[k];
      }
    }
  }
  mark(ctx, "batch_grouped");
  // large instances: the single-system solver, one after the other (each
  // fills the device by itself)
  for (int i : rest) {
    Matrix* A = B->mats[i];
    const int64_t off = B->h_inst[i].off;
    GT_CUDA(ctx, cudaMemsetAsync(x + off, 0, sizeof(double) * A->nbrows * A->bs, ctx->stream));
    // a matrix of another context solves on that context's stream: b and x
    // (written on this one) are complete first; solve() returns synchronised
    if (A->ctx != ctx) GT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int s = solve(A, b + off, x + off, rtol, maxit, mode, &info[i]);
    if (s != GT_OK && s != GT_ERR_NOT_CONVERGED) return s;
    if (s == GT_ERR_NOT_CONVERGED) status = s;
  }
  mark(ctx, "batch_large");
  if (infos)
    for (int i = 0; i < ni; i++) infos[i] = info[i];
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
    if (!A || A->ctx->device != ctx->device || (A->bs != 1 && A->bs != 3)) {
      delete B;
      return set_error(ctx, GT_ERR_INVALID,
                       "batch: matrices must have block size 1 or 3 and be on this context's device");
    }
    int s = find_diag(A);
    // a matrix of another context (assembled on another stream): its
    // diagonal positions are complete before this context's kernels read them
    if (s == GT_OK && A->ctx != ctx && cudaStreamSynchronize(A->ctx->stream) != cudaSuccess)
      s = set_error(ctx, GT_ERR_CUDA, "batch: synchronising a matrix's context failed");
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
    in.bs = A->bs;
    off += A->nbrows * A->bs;
    B->h_inst.push_back(in);
    B->mats.push_back(A);
  }
  classify(B);  // largest small instances first: the queue then balances the CTAs
  B->ntot = off;
  int s = dalloc(ctx, &B->d_inst, n);
  if (s == GT_OK) s = copy_in(ctx, B->d_inst, B->h_inst.data(), n);
  if (s == GT_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess) s = GT_ERR_CUDA;
  if (s != GT_OK) {
    gt_batch_destroy(B);
    return s;
  }
  *out = B;
  return GT_OK;
}

int gt_batch_set_lanes(gt_batch* B, int lanes) {
  if (!B || (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8)) return GT_ERR_INVALID;
  B->G = lanes;
  return GT_OK;
}

int gt_batch_set_small_rows(gt_batch* B, int64_t rows) {
  if (!B || rows < 0 || rows > kSmallRows) return GT_ERR_INVALID;
  B->small_rows = rows;
  classify(B);
  return GT_OK;
}

int gt_batch_info(const gt_batch* B, int64_t* info) {
  if (!B || !info) return GT_ERR_INVALID;
  info[0] = B->n;
  info[1] = B->ntot;
  info[2] = (int64_t)B->small.size();
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
  delete B;
  return GT_OK;
}

}  // extern "C"
