// gt_assembly.cu -- sparsity construction, per-cell integration and the
// deterministic CSR scatter.
//
// Pipeline of one assemble_matrix call (reference: src/problems.jl:319-350
// -> allocate_matrix counting pass src/assembly.jl:119-153, the generated
// cell loop src/compiler.jl:1865-1917 with contribute! src/assembly.jl:
// 189-208, and the COO->CSC compress src/assembly.jl:571-575):
//   1. incidence: block row (free node dof) -> sorted list of (cell, local
//      node) that touch it  [k_inc_count, scan, k_inc_fill, k_inc_sort]
//      (k_inc_sort: one warp per row, bitonic sort in shared memory)
//   2. pattern: per block row, the sorted union of the free node dofs of its
//      cells  [k_pattern<count>, scan, k_pattern<fill>]  == the reference's
//      sorted, duplicate-free CSC (the forms are symmetric, CSR == CSC)
//   3. element matrices: FP64 Jacobian / inverse / determinant per
//      quadrature point, element matrix in T (FP64 or FP32)  [k_elements]
//   4. scatter: each block row is owned by one thread group that sums the
//      contributions of its cells in ascending cell order -- the order in
//      which the reference's COO->CSC conversion sums duplicates -- and
//      writes the row once.  No atomics on values: bitwise deterministic.
#include <climits>
#include <cstring>
#include <type_traits>

#include "gt_internal.cuh"
#include "gt_dfloat.cuh"
#include "gt_refcell.cuh"

namespace gt {

static inline Ctx* ctx_of(const Space* sp) { return sp->mesh->ctx; }

// ---------------------------------------------------------------------------
// reference tabulation (quadrature + shape functions), built on the device
// quadrature: tensor Gauss-Legendre, ceil((deg+1)/2) points per direction,
// first index fastest (src/quadrature.jl:78-106); tetrahedron: 4-point Strang
// rule (src/quadrature.jl:512-529).  Shape functions: tensor-product Lagrange
// on equispaced nodes (the reference builds the same basis from monomials
// and a Vandermonde inverse, src/space.jl:942-970).
// ---------------------------------------------------------------------------
struct TabLayout {
  int D, nlv, nn, nq;
  int off_w, off_gg, off_sv, off_sg;
  int off_k;  // 48 doubles of per-reference-cell quadrature sums (P1 path): 22 FP64 sums, then FP32-pair splits
  int off_gv;  // geometry shape values at the points (nq x nlv), past the kernels' staged part
  int total;
};
inline TabLayout tab_layout(int ctype, int order) {
  TabLayout L{};
  L.D = ctype == GT_QUAD4 ? 2 : 3;
  L.nlv = ctype == GT_QUAD4 ? 4 : (ctype == GT_HEX8 ? 8 : 4);
  L.nn = space_nodes(ctype, order);
  int n1 = ctype == GT_TET4 ? 0 : order + 1;  // Gauss points per direction for degree 2*order
  // tets: the 4-point degree-2 rule (P1) or the 11-point degree-4 rule (P2)
  L.nq = ctype == GT_TET4 ? (order == 2 ? 11 : 4) : (L.D == 2 ? n1 * n1 : n1 * n1 * n1);
  L.off_w = 0;
  L.off_gg = L.nq;
  L.off_sv = L.off_gg + L.nq * L.nlv * L.D;
  L.off_sg = L.off_sv + L.nq * L.nn;
  L.off_k = L.off_sg + L.nq * L.nn * L.D;
  L.off_gv = L.off_k + 48;
  L.total = L.off_gv + L.nq * L.nlv;
  return L;
}

__device__ void lagrange1d(int order, double x, double* v, double* dv) {
  if (order == 1) {
    v[0] = 1.0 - x; v[1] = x; dv[0] = -1.0; dv[1] = 1.0;
  } else {
    v[0] = 2.0 * (x - 0.5) * (x - 1.0);
    v[1] = -4.0 * x * (x - 1.0);
    v[2] = 2.0 * x * (x - 0.5);
    dv[0] = 4.0 * x - 3.0; dv[1] = -8.0 * x + 4.0; dv[2] = 4.0 * x - 1.0;
  }
}

// 1/d for d != 0 from the hardware reciprocal approximation (PTX
// rcp.approx.ftz.f64) refined by two Newton-Raphson steps r <- r + r (1 - d r)
// (each squares the relative error): within a few ulp of the rounded
// quotient, in four FP64 FMAs instead of the correctly rounded division's
// longer sequence -- the element kernels are bound by FP64 issue slots.
__device__ __forceinline__ double recip_nr2(double d) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  e = fma(-d, r, 1.0);
  return fma(r, e, r);
}

__global__ void k_tabulate(int ctype, int order, TabLayout L, double* tab) {
  int q = threadIdx.x;
  if (q >= L.nq) return;
  double x[3] = {0, 0, 0}, w;
  if (ctype == GT_TET4 && order == 2) {
    // Keast's 11-point rule of degree 4 on the unit tetrahedron (the
    // reference's strang_quadrature_4, src/quadrature.jl:554-590): the
    // centroid (negative weight), the 4 points (11/14, 1/14, 1/14) and
    // permutations plus (1/14,1/14,1/14), and the 6 points with two
    // coordinates (1 + sqrt(5/14))/4 and one (1 - sqrt(5/14))/4 or the reverse
    const double r = sqrt(5.0 / 14.0), a = 0.25 * (1.0 + r), b = 0.25 * (1.0 - r);
    const double f = 11.0 / 14.0, g = 1.0 / 14.0;
    const double P[11][3] = {{0.25, 0.25, 0.25}, {f, g, g}, {g, f, g}, {g, g, f}, {g, g, g}, {a, a, b},
                             {a, b, a},          {a, b, b}, {b, a, a}, {b, a, b}, {b, b, a}};
    for (int d = 0; d < 3; d++) x[d] = P[q][d];
    w = q == 0 ? -74.0 / 5625.0 : (q < 5 ? 343.0 / 45000.0 : 56.0 / 2250.0);
  } else if (ctype == GT_TET4) {
    const double a = 0.5854101966249685, b = 0.1381966011250105;
    x[0] = x[1] = x[2] = b;
    if (q > 0) x[q - 1] = a;
    w = 1.0 / 24.0;
  } else {
    int n1 = order + 1;
    double g[3], gw[3];
    if (n1 == 2) {
      double s = 0.5 / sqrt(3.0);
      g[0] = 0.5 - s; g[1] = 0.5 + s; gw[0] = gw[1] = 0.5;
    } else {
      double s = 0.5 * sqrt(0.6);
      g[0] = 0.5 - s; g[1] = 0.5; g[2] = 0.5 + s;
      gw[0] = 5.0 / 18.0; gw[1] = 8.0 / 18.0; gw[2] = 5.0 / 18.0;
    }
    int i[3] = {q % n1, (q / n1) % n1, q / (n1 * n1)};
    w = 1.0;
    for (int d = 0; d < L.D; d++) { x[d] = g[i[d]]; w *= gw[i[d]]; }
  }
  tab[L.off_w + q] = w;
  // geometry map gradients (P1 / Q1)
  if (ctype == GT_TET4) {
    const double gr[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    const double v[4] = {1.0 - x[0] - x[1] - x[2], x[0], x[1], x[2]};  // barycentric coordinates
    for (int n = 0; n < 4; n++) {
      tab[L.off_gv + q * 4 + n] = v[n];
      for (int d = 0; d < 3; d++) tab[L.off_gg + (q * 4 + n) * 3 + d] = gr[n][d];
    }
    if (order == 1) {
      for (int n = 0; n < 4; n++) {
        tab[L.off_sv + q * 4 + n] = v[n];
        for (int d = 0; d < 3; d++) tab[L.off_sg + (q * 4 + n) * 3 + d] = gr[n][d];
      }
      return;
    }
    // P2 in barycentric form: vertex i -> l_i (2 l_i - 1), edge (i, j) ->
    // 4 l_i l_j, at the node order of the exponents (first index fastest)
    const int vi[10] = {0, -1, 1, -1, -1, 2, -1, -1, -1, 3};
    const int ei[10][2] = {{0, 0}, {0, 1}, {0, 0}, {0, 2}, {1, 2}, {0, 0}, {0, 3}, {1, 3}, {2, 3}, {0, 0}};
    for (int n = 0; n < 10; n++) {
      double val, g[3];
      if (vi[n] >= 0) {
        const int i = vi[n];
        val = v[i] * (2.0 * v[i] - 1.0);
        for (int d = 0; d < 3; d++) g[d] = (4.0 * v[i] - 1.0) * gr[i][d];
      } else {
        const int i = ei[n][0], j = ei[n][1];
        val = 4.0 * v[i] * v[j];
        for (int d = 0; d < 3; d++) g[d] = 4.0 * (v[j] * gr[i][d] + v[i] * gr[j][d]);
      }
      tab[L.off_sv + q * 10 + n] = val;
      for (int d = 0; d < 3; d++) tab[L.off_sg + (q * 10 + n) * 3 + d] = g[d];
    }
    return;
  }
  double v1[3][3], d1[3][3];
  for (int d = 0; d < L.D; d++) lagrange1d(1, x[d], v1[d], d1[d]);
  for (int n = 0; n < L.nlv; n++) {
    double g = 1.0;
    for (int e = 0; e < L.D; e++) g *= v1[e][(n >> e) & 1];
    tab[L.off_gv + q * L.nlv + n] = g;
  }
  for (int n = 0; n < L.nlv; n++)
    for (int d = 0; d < L.D; d++) {
      double g = 1.0;
      for (int e = 0; e < L.D; e++) {
        int bit = (n >> e) & 1;
        g *= (e == d) ? d1[e][bit] : v1[e][bit];
      }
      tab[L.off_gg + (q * L.nlv + n) * L.D + d] = g;
    }
  double vk[3][3], dk[3][3];
  for (int d = 0; d < L.D; d++) lagrange1d(order, x[d], vk[d], dk[d]);
  int m = order + 1;
  for (int n = 0; n < L.nn; n++) {
    int e[3] = {n % m, (n / m) % m, n / (m * m)};
    double p = 1.0;
    for (int d = 0; d < L.D; d++) p *= vk[d][e[d]];
    tab[L.off_sv + q * L.nn + n] = p;
    for (int d = 0; d < L.D; d++) {
      double g = 1.0;
      for (int d2 = 0; d2 < L.D; d2++) g *= (d2 == d) ? dk[d2][e[d2]] : vk[d2][e[d2]];
      tab[L.off_sg + (q * L.nn + n) * L.D + d] = g;
    }
  }
}

static int get_tab(Ctx* ctx, int ctype, int order, double** tab, TabLayout* L) {
  *L = tab_layout(ctype, order);
  GT_TRY(dalloc(ctx, tab, L->total));
  k_tabulate<<<GT_KC(ctx, 1), 32, 0, ctx->stream>>>(ctype, order, *L, *tab);
  GT_LAUNCH(ctx, "k_tabulate");
  return GT_OK;
}

// ---------------------------------------------------------------------------
// 1. incidence
// ---------------------------------------------------------------------------
// count the incidences of every free node and give each (cell, node) entry
// its rank among the entries of its node.  Entries of one warp that name the
// same node (consecutive cells share nodes) take one atomic for the group
// (the atomics, one L2 round trip each, bound this pass).  Ranks follow the
// atomics' order; the sparsity pass sorts every row's list afterwards.
__global__ void k_inc_count(const int32_t* __restrict__ cnd, int64_t n, int32_t* __restrict__ cnt,
                            int32_t* __restrict__ rank) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // warp-uniform loop: every lane takes part in the match below
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += stride) {
    const int64_t i = i0 + lane;
    const int32_t d = i < n ? __ldg(cnd + i) : 0;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    int32_t base = 0;
    if (lane == leader && d > 0) base = atomicAdd(&cnt[d - 1], __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (d > 0) rank[i] = base + __popc(peers & ((1u << lane) - 1u));
  }
}
__global__ void k_inc_fill(const int32_t* __restrict__ cnd, int64_t n, const int64_t* __restrict__ ptr,
                           const int32_t* __restrict__ rank, int32_t* __restrict__ inc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t d = __ldg(cnd + i);
    if (d > 0) inc[__ldg(ptr + d - 1) + __ldg(rank + i)] = (int32_t)i;  // cell * nn + local node
  }
}
// The incidence of a matrix whose rows the row-per-thread count pass takes
// (P1/Q1, at most kIncBucket incidences per row), in one pass: every entry
// takes its position among its node's entries as in k_inc_count and is
// written straight into its row's bucket of kIncBucket slots, so neither
// the ranks nor a fill pass are needed.  Entries beyond a bucket are only
// counted; the count pass then finds the row too long, and the incidence is
// rebuilt by k_inc_count + k_inc_fill for the warp-per-row kernel.
constexpr int kIncBucket = 32;
__global__ void k_inc_place(const int32_t* __restrict__ cnd, int64_t n, int32_t* __restrict__ cnt,
                            int32_t* __restrict__ bucket) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += stride) {
    const int64_t i = i0 + lane;
    const int32_t d = i < n ? __ldg(cnd + i) : 0;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    int32_t base = 0;
    if (lane == leader && d > 0) base = atomicAdd(&cnt[d - 1], __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    const int32_t pos = base + __popc(peers & ((1u << lane) - 1u));
    if (d > 0 && pos < kIncBucket) bucket[(int64_t)(d - 1) * kIncBucket + pos] = (int32_t)i;
  }
}

// sort each row's incidences ascending (= by cell): one warp per row,
// bitonic sort in shared memory (icap slots per warp)
// ascending bitonic sort of buf[0..P) (P a power of two >= 32) by one warp
__device__ __forceinline__ void warp_bitonic_sort(int32_t* buf, int P, int lane) {
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < P; i += 32) {
        int ixj = i ^ j;
        if (ixj > i) {
          int32_t a = buf[i], b = buf[ixj];
          bool up = (i & k) == 0;
          if ((a > b) == up) { buf[i] = b; buf[ixj] = a; }
        }
      }
      __syncwarp();
    }
  }
}

__global__ void k_inc_sort(const int64_t* __restrict__ ptr, int32_t* __restrict__ inc, int64_t nrows, int icap) {
  extern __shared__ int32_t s_ibuf[];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t* buf = s_ibuf + w * icap;
  int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + w;
  if (r >= nrows) return;
  int64_t b = ptr[r];
  int n = (int)(ptr[r + 1] - b);
  int P = 32;
  while (P < n) P <<= 1;
  for (int i = lane; i < P; i += 32) buf[i] = i < n ? inc[b + i] : INT_MAX;
  __syncwarp();
  warp_bitonic_sort(buf, P, lane);
  for (int i = lane; i < n; i += 32) inc[b + i] = buf[i];
}

static int max_diff(Ctx* ctx, const int64_t* ptr, int64_t n, int32_t* out);

int build_incidence(Ctx* ctx, const Space* sp, int64_t** inc_ptr, int32_t** inc, int64_t* ninc, bool sort) {
  return build_incidence_arr(ctx, sp->cell_ndofs, sp->mesh->ncells * sp->nn, sp->nfree_nodes, inc_ptr, inc, ninc, sort);
}

// the incidence lists of any array of n node-level DOF ids (>0 free): row r
// lists the positions i with dofs[i] == r + 1
int build_incidence_arr(Ctx* ctx, const int32_t* dofs, int64_t n, int64_t nrows, int64_t** inc_ptr, int32_t** inc,
                        int64_t* ninc, bool sort) {
  cudaStream_t st = ctx->stream;
  int32_t *cnt = nullptr, *rank = nullptr;
  GT_TRY(dalloc(ctx, &cnt, nrows + 1));
  GT_TRY(dalloc(ctx, &rank, n > 0 ? n : 1));
  GT_TRY(dalloc(ctx, inc_ptr, nrows + 1));
  GT_TRY(dalloc(ctx, inc, n));  // upper bound: every (cell, node) free
  GT_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (nrows + 1), st));
  if (n > 0) k_inc_count<<<GT_KC(ctx, grid_for(n, 256)), 256, 0, st>>>(dofs, n, cnt, rank);
  GT_LAUNCH(ctx, "k_inc_count");
  GT_TRY(exclusive_scan_i64(ctx, cnt, *inc_ptr, nrows));
  if (n > 0) k_inc_fill<<<GT_KC(ctx, grid_for(n, 256)), 256, 0, st>>>(dofs, n, *inc_ptr, rank, *inc);
  GT_LAUNCH(ctx, "k_inc_fill");
  *ninc = -1;  // not read back: the sparsity pass knows the row extents
  if (sort) {
    int32_t maxinc = 0;
    GT_TRY(max_diff(ctx, *inc_ptr, nrows, &maxinc));
    int icap = 32;
    while (icap < maxinc) icap <<= 1;
    if (icap > 4096) return set_error(ctx, GT_ERR_UNSUPPORTED, "a DOF touches too many cells");
    int warps = 8;
    size_t smem = (size_t)warps * icap * sizeof(int32_t);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_inc_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (nrows > 0)
      k_inc_sort<<<GT_KC(ctx, grid_for(nrows, warps)), warps * 32, smem, st>>>(*inc_ptr, *inc, nrows, icap);
    GT_LAUNCH(ctx, "k_inc_sort");
  }
  dfree(ctx, cnt);
  dfree(ctx, rank);
  return GT_OK;
}

// ---------------------------------------------------------------------------
// 2. pattern
// ---------------------------------------------------------------------------
// ascending bitonic sort of NK (16 or 32) keys held one per lane (register
// shuffles).  In stage (k = 2^a, j = 2^b) a lane keeps the larger key iff
// bits a and b of its lane index differ, i.e. bit b of lane ^ (lane >> (a-b));
// the shifted indices are formed once, so a stage is a shuffle, a bit
// test and a min/max.  With NK = 16 both half-warps sort their own lanes
// (lanes 0..15 ascending).
template <int NK>
__device__ __forceinline__ int32_t warp_sort(int32_t v, int lane) {
  const int x[6] = {0, lane ^ (lane >> 1), lane ^ (lane >> 2), lane ^ (lane >> 3), lane ^ (lane >> 4), lane};
#pragma unroll
  for (int a = 1; (1 << a) <= NK; a++)
#pragma unroll
    for (int b = a - 1; b >= 0; b--) {
      const int32_t o = __shfl_xor_sync(0xffffffffu, v, 1 << b);
      v = (x[a - b] >> b) & 1 ? max(v, o) : min(v, o);
    }
  return v;
}

// Per block row: the sorted union of the free node DOFs of its cells.
// One warp per row.  The row's incidences are sorted ascending (= by cell;
// the count pass writes them back, which fixes the scatter's summation
// order) and held one per lane.  The row's own DOF (block row r is node
// r + 1, present in every incident cell) goes in first; the other nodes of
// the incident cells follow in rounds of 32 candidates.  In a round, lanes
// holding the same key elect one leader (match.any), so a shared-memory hash
// set (linear probing, empty = -1) sees each key at most once per round and
// its compare-and-swaps never serialise on one address; a leader that
// inserted appends its key to the row's list (ballot + prefix count).  The
// count pass counts the distinct keys and, for rows of at most S columns,
// sorts them (register shuffles for <= 32 keys, shared-memory bitonic sort
// above) into the row's slot of S entries; the fill pass copies those slots
// and runs the hash again only for longer rows.
template <int NN, int S, bool FILL>
__global__ void __launch_bounds__(256) k_pattern(const int64_t* __restrict__ inc_ptr, int32_t* __restrict__ inc,
                                                 const int32_t* __restrict__ cnd, int64_t nrows, int hcap, int icap,
                                                 int32_t* __restrict__ rowcnt, const int64_t* __restrict__ rowptr,
                                                 int32_t* __restrict__ colind, int32_t* __restrict__ slots,
                                                 uint8_t* __restrict__ small, int32_t* maxrow, uint32_t* err) {
  extern __shared__ int32_t s_buf[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t* tab = s_buf + (size_t)w * (hcap + 2 * icap);  // hash set
  int32_t* ibuf = tab + hcap;                            // sorted incidences of rows with more than 32
  int32_t* keys = ibuf + icap;                           // the row's distinct columns, insertion order
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + w;
  if (r >= nrows) return;
  if (FILL && small[r]) {
    // the count pass already wrote this row's sorted columns to its slot
    int64_t o = rowptr[r];
    int n = (int)(rowptr[r + 1] - o);
    for (int i = lane; i < n; i += 32) colind[o + i] = slots[r * S + i];
    return;
  }
  const int64_t ib = inc_ptr[r];
  const int ninc = (int)(inc_ptr[r + 1] - ib);
  const int ncand = ninc * NN;
  if (ncand + (ncand >> 2) > hcap || ncand > icap) {
    if (lane == 0) { atomicOr(err, DEV_ERR_ROW_CAP); if (!FILL) { rowcnt[r] = 0; small[r] = 1; } }
    return;
  }
  for (int i = lane; i < (hcap >> 2); i += 32) reinterpret_cast<int4*>(tab)[i] = make_int4(-1, -1, -1, -1);
  int32_t myinc = INT_MAX;  // lane k: the k-th incidence (rows of at most 32)
  if (ninc <= 32) {
    const int32_t u = lane < ninc ? inc[ib + lane] : INT_MAX;
    if (FILL) {
      myinc = u;  // sorted by the count pass
    } else {
      myinc = ninc <= 16 ? warp_sort<16>(u, lane) : warp_sort<32>(u, lane);
      if (lane < ninc) inc[ib + lane] = myinc;
    }
  } else if (!FILL) {
    int P2 = 64;
    while (P2 < ninc) P2 <<= 1;
    for (int i = lane; i < P2; i += 32) ibuf[i] = i < ninc ? inc[ib + i] : INT_MAX;
    __syncwarp();
    warp_bitonic_sort(ibuf, P2, lane);
    for (int i = lane; i < ninc; i += 32) inc[ib + i] = ibuf[i];
  } else {
    for (int i = lane; i < ninc; i += 32) ibuf[i] = inc[ib + i];
  }
  __syncwarp();
  const unsigned hmask = (unsigned)hcap - 1u;
  const unsigned lt = (1u << lane) - 1u;
  if (lane == 0 && ninc > 0) {
    tab[((unsigned)r * 2654435761u) & hmask] = (int32_t)r;
    keys[0] = (int32_t)r;
  }
  int total = ninc > 0 ? 1 : 0;
  __syncwarp();
  bool lost = false;  // a probe sequence ran through the whole table (cannot happen: a slot stays free)
  const int nround = (ncand + 31) >> 5;
  for (int t = 0; t < nround; t++) {
    const int i = t * 32 + lane;
    const int k = i / NN, b = i - k * NN;
    int32_t e = 0;
    if (ninc <= 32) e = __shfl_sync(0xffffffffu, myinc, k & 31);
    else if (i < ncand) e = ibuf[k];
    int32_t key = -1;
    if (i < ncand) {
      const int32_t c = e / NN;
      if (b != e - c * NN) {
        const int32_t d = __ldg(cnd + (int64_t)c * NN + b);
        if (d > 0) key = d - 1;
      }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    bool ins = false;
    if (key >= 0 && (peers & lt) == 0) {
      unsigned h = ((unsigned)key * 2654435761u) & hmask;
      bool done = false;
      for (unsigned probe = 0; probe <= hmask; probe++) {
        const int32_t old = atomicCAS(&tab[h], -1, key);
        if (old == -1) { ins = true; done = true; break; }
        if (old == key) { done = true; break; }
        h = (h + 1) & hmask;
      }
      lost |= !done;
    }
    const unsigned m = __ballot_sync(0xffffffffu, ins);
    if (ins) keys[total + __popc(m & lt)] = key;
    total += __popc(m);
  }
  if (__any_sync(0xffffffffu, lost)) {
    if (lane == 0) { atomicOr(err, DEV_ERR_HASH_FULL); if (!FILL) { rowcnt[r] = 0; small[r] = 1; } }
    return;
  }
  __syncwarp();
  if (!FILL) {
    if (lane == 0) {
      rowcnt[r] = total;
      // the running maximum changes rarely: skip the same-address atomic
      // (one per row otherwise, serialised in one L2 slice) when not above it
      if (total > __ldcg(maxrow)) atomicMax(maxrow, total);
      small[r] = total <= S;
    }
    if (total > S) return;
  }
  // sort the distinct keys (total <= ncand <= icap) and write them to the
  // row's slot (count pass) or to colind (fill pass)
  if (total <= 32) {
    const int32_t u = lane < total ? keys[lane] : INT_MAX;
    const int32_t v = total <= 16 ? warp_sort<16>(u, lane) : warp_sort<32>(u, lane);
    if (lane < total) {
      if (FILL) colind[rowptr[r] + lane] = v;
      else slots[r * S + lane] = v;
    }
    return;
  }
  int P = 64;
  while (P < total) P <<= 1;
  for (int i = total + lane; i < P; i += 32) keys[i] = INT_MAX;
  __syncwarp();
  warp_bitonic_sort(keys, P, lane);
  if (FILL) {
    int64_t o = rowptr[r];
    for (int i = lane; i < total; i += 32) colind[o + i] = keys[i];
  } else {
    for (int i = lane; i < total; i += 32) slots[r * S + i] = keys[i];
  }
}

// The count pass with one thread per block row, for rows of at most 32
// incidences and 32 columns (P1 tetrahedra, Q1 quadrilaterals and hexahedra):
// the thread sorts its incidences by insertion and builds its sorted column
// list by binary search and insertion, both in shared memory interleaved
// across the block's threads (element k of thread t at k * blockDim + t).
// A row with more than 32 incidences or 32 columns sets *redo.  With bucket
// the incidences are read from the row's bucket (k_inc_place) and the
// sorted list is written to the row's CSR range.
// A warp then works on 32 rows at once instead of one, which cuts the warp
// instructions per row several times over the warp-per-row kernel (whose
// sorts, rounds and compaction are per-warp costs).  Same results: the
// row's incidences ascending, its distinct free columns ascending.  After a
// *redo the warp kernel recounts every row.
// C16: the space's DOF spread is below 2^15, so every column differs from
// its row by less than 2^15 and the list holds column - row in 16 bits:
// 192 instead of 256 bytes of shared memory per thread, 9 instead of 6
// blocks per SM (the pass is bound by shared-memory latency, not bandwidth).
constexpr int kRowsMI = 32, kRowsS = 32;
static_assert(kIncBucket == kRowsMI, "a bucket holds the incidences the row-per-thread pass takes");
template <int NN, bool C16>
__global__ void __launch_bounds__(128) k_pattern_rows(const int64_t* __restrict__ inc_ptr, int32_t* __restrict__ inc,
                                                      const int32_t* __restrict__ cnd, int64_t nrows,
                                                      int32_t* __restrict__ rowcnt, int32_t* __restrict__ slots,
                                                      uint8_t* __restrict__ small, int32_t* maxrow, int32_t* redo,
                                                      const int32_t* __restrict__ bucket) {
  extern __shared__ int32_t s_rows[];
  using CT = typename std::conditional<C16, int16_t, int32_t>::type;
  const int T = blockDim.x, tid = threadIdx.x;
  int32_t* I = s_rows + tid;                                      // incidences, I[k * T]
  CT* Cl = reinterpret_cast<CT*>(s_rows + kRowsMI * T) + tid;     // columns (- row with C16), Cl[k * T]
  const int64_t r = blockIdx.x * (int64_t)T + tid;
  const int32_t cbase = C16 ? (int32_t)r : 0;
  if (r >= nrows) return;
  const int64_t ib = inc_ptr[r];
  const int ninc = (int)(inc_ptr[r + 1] - ib);
  if (ninc > kRowsMI) {  // more incidences than the buffer: the warp kernel recounts
    *redo = 1;
    rowcnt[r] = 0;
    small[r] = 0;
    return;
  }
  // the row's incidences, sorted by insertion in I: from its bucket
  // (k_inc_place; 16-byte aligned, so all of it is loaded at once into I and
  // sorted in place) or from its CSR list
  if (bucket) {
    const int4* b4 = reinterpret_cast<const int4*>(bucket + r * kIncBucket);
    int4 v[kIncBucket / 4];
#pragma unroll
    for (int q = 0; q < kIncBucket / 4; q++)
      if (4 * q < ninc) v[q] = __ldg(b4 + q);
#pragma unroll
    for (int q = 0; q < kIncBucket / 4; q++)
      if (4 * q < ninc) {
        I[(4 * q) * T] = v[q].x;
        I[(4 * q + 1) * T] = v[q].y;
        I[(4 * q + 2) * T] = v[q].z;
        I[(4 * q + 3) * T] = v[q].w;
      }
    for (int k = 1; k < ninc; k++) {
      const int32_t x = I[k * T];
      int j = k;
      while (j > 0 && I[(j - 1) * T] > x) {
        I[j * T] = I[(j - 1) * T];
        j--;
      }
      I[j * T] = x;
    }
  } else {
    for (int k = 0; k < ninc; k++) {
      const int32_t x = inc[ib + k];
      int j = k;
      while (j > 0 && I[(j - 1) * T] > x) {
        I[j * T] = I[(j - 1) * T];
        j--;
      }
      I[j * T] = x;
    }
  }
  for (int k = 0; k < ninc; k++) inc[ib + k] = I[k * T];
  int n = 0;
  bool over = false;
  if (ninc > 0) {
    Cl[0] = (CT)((int32_t)r - cbase);  // the row's own DOF (block row r is node r + 1)
    n = 1;
  }
  // the next incidence's node DOFs are loaded while the current ones are
  // inserted (P1: one 16-byte load per incidence)
  int4 nxt = make_int4(0, 0, 0, 0);
  if (NN == 4 && ninc > 0) nxt = __ldg(reinterpret_cast<const int4*>(cnd) + I[0] / NN);
  // the node DOFs of the previous PV incidences (all already in the list):
  // a candidate equal to one of them is a known duplicate and skips the
  // search.  Incidences are visited by ascending cell, and neighbouring cells
  // share most of their nodes (on the P1 benchmark mesh this filter takes out
  // about half of the searches)
  constexpr int PV = NN <= 4 ? 2 : (NN <= 8 ? 1 : 0);
  int32_t prev[PV > 0 ? PV : 1][NN];
#pragma unroll
  for (int u = 0; u < PV; u++)
#pragma unroll
    for (int b = 0; b < NN; b++) prev[u][b] = 0;
  for (int k = 0; k < ninc; k++) {
    const int32_t e = I[k * T];
    const int32_t c = e / NN, self = e - c * NN;
    int32_t d[NN];
    if constexpr (NN == 4) {
      const int4 q = nxt;
      if (k + 1 < ninc) nxt = __ldg(reinterpret_cast<const int4*>(cnd) + I[(k + 1) * T] / NN);
      d[0] = q.x; d[1] = q.y; d[2] = q.z; d[3] = q.w;
    } else if constexpr (NN == 8) {
      const int4 q0 = __ldg(reinterpret_cast<const int4*>(cnd) + 2 * (int64_t)c);
      const int4 q1 = __ldg(reinterpret_cast<const int4*>(cnd) + 2 * (int64_t)c + 1);
      d[0] = q0.x; d[1] = q0.y; d[2] = q0.z; d[3] = q0.w; d[4] = q1.x; d[5] = q1.y; d[6] = q1.z; d[7] = q1.w;
    } else {
#pragma unroll
      for (int b = 0; b < NN; b++) d[b] = __ldg(cnd + (int64_t)c * NN + b);
    }
#pragma unroll
    for (int b = 0; b < NN; b++) {
      if (b == self || d[b] <= 0) continue;
      bool known = false;
#pragma unroll
      for (int u = 0; u < PV; u++)
#pragma unroll
        for (int q = 0; q < NN; q++) known |= prev[u][q] == d[b];
      if (known) continue;
      const int32_t key = d[b] - 1 - cbase;
      int lo = 0, hi = n;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (Cl[mid * T] < key) lo = mid + 1;
        else hi = mid;
      }
      if (lo < n && Cl[lo * T] == key) continue;
      if (n == kRowsS) {
        over = true;
        continue;
      }
      for (int j = n; j > lo; j--) Cl[j * T] = Cl[(j - 1) * T];
      Cl[lo * T] = (CT)key;
      n++;
    }
    if constexpr (PV > 0) {
#pragma unroll
      for (int u = PV - 1; u > 0; u--)
#pragma unroll
        for (int b = 0; b < NN; b++) prev[u][b] = prev[u - 1][b];
#pragma unroll
      for (int b = 0; b < NN; b++) prev[0][b] = d[b];
    }
  }
  if (over) {
    *redo = 1;
    rowcnt[r] = 0;
    small[r] = 0;
    return;
  }
  rowcnt[r] = n;
  small[r] = 1;
  for (int k = 0; k < n; k++) slots[r * kRowsS + k] = (int32_t)Cl[k * T] + cbase;
  if (n > __ldcg(maxrow)) atomicMax(maxrow, n);
}

// colind of the rows whose sorted columns the count pass left in their slot
// of S entries: four lanes per row, each copying a quarter of the row with
// 16-byte slot loads (slots are 16-byte aligned), all loads in flight
template <int S>
__global__ void k_copy_slots(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ slots, int64_t nrows,
                             int32_t* __restrict__ colind) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t r = t >> 2;
  int q = (int)(t & 3);
  if (r >= nrows) return;
  const int64_t o = rowptr[r];
  const int n = (int)(rowptr[r + 1] - o);
  constexpr int V4 = S / 16;  // int4 loads per lane
  const int4* src = reinterpret_cast<const int4*>(slots + r * S) + q * V4;
  int4 v[V4];
#pragma unroll
  for (int k = 0; k < V4; k++)
    if ((q * V4 + k) * 4 < n) v[k] = __ldg(src + k);
#pragma unroll
  for (int k = 0; k < V4; k++) {
    const int b = (q * V4 + k) * 4;
    if (b < n) colind[o + b] = v[k].x;
    if (b + 1 < n) colind[o + b + 1] = v[k].y;
    if (b + 2 < n) colind[o + b + 2] = v[k].z;
    if (b + 3 < n) colind[o + b + 3] = v[k].w;
  }
}

__global__ void k_max_diff(const int64_t* ptr, int64_t n, int32_t* out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int32_t v = 0;
  if (i < n) v = (int32_t)(ptr[i + 1] - ptr[i]);
  for (int o = 16; o; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, v);
}

static int max_diff(Ctx* ctx, const int64_t* ptr, int64_t n, int32_t* out) {
  int32_t* d = nullptr;
  GT_TRY(dalloc(ctx, &d, 1));
  GT_CUDA(ctx, cudaMemsetAsync(d, 0, sizeof(int32_t), ctx->stream));
  if (n > 0) k_max_diff<<<GT_KC(ctx, grid_for(n, 256)), 256, 0, ctx->stream>>>(ptr, n, d);
  GT_LAUNCH(ctx, "k_max_diff");
  GT_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scratch[8], d, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  GT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  memcpy(out, &ctx->h_scratch[8], sizeof(int32_t));
  dfree(ctx, d);
  return GT_OK;
}

// The last cell among the incidences of each row chunk (rows
// nrows*k/K .. nrows*(k+1)/K, K = kRowChunks): after the count pass every
// row's list is sorted, so a row's last incidence holds its last cell.  Per
// warp, one max reduction and one atomicMax for each chunk its rows touch.
__global__ void k_chunk_last(const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc, int64_t nrows,
                             int nn, int32_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); r0 < nrows; r0 += stride) {
    const int64_t r = r0 + lane;
    const bool in = r < nrows;
    int32_t v = -1;
    int k = 0;
    if (in) {
      const int64_t b = inc_ptr[r], e = inc_ptr[r + 1];
      if (e > b) v = inc[e - 1] / nn;
      k = (int)(((r + 1) * kRowChunks - 1) / nrows);  // the chunk whose range holds r
    }
    unsigned todo = __ballot_sync(0xffffffffu, in);
    while (todo) {
      const int src = __ffs(todo) - 1;
      const int kk = __shfl_sync(0xffffffffu, k, src);
      const bool mine = in && k == kk;
      int32_t m = mine ? v : -1;
#pragma unroll
      for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
      if (lane == src && m >= 0) atomicMax(out + kk, m);
      todo &= ~__ballot_sync(0xffffffffu, mine);
    }
  }
}

// bucket (optional): the incidences were placed by k_inc_place (row r's in
// bucket[r * kIncBucket ...]); A->inc then only receives the sorted lists
// want_last: also find each row chunk's last cell (A->chunk_last)
template <int NN>
static int launch_pattern(Matrix* A, int32_t maxinc, const int32_t* bucket, bool want_last) {
  // slot width of the count pass: P1/Q1/Q2-quad rows have <= 27 columns,
  // Q2-hex rows up to 125
  constexpr int S = NN >= 10 ? 128 : 32;  // P2-tet rows: up to ~70 columns
  const Space* sp = A->space;
  Ctx* ctx = sp->mesh->ctx;
  cudaStream_t st = ctx->stream;
  int64_t nrows = A->nbrows;
  // hash table: load factor <= 0.8 even if every candidate were distinct;
  // ibuf holds the row's incidences, then the compacted keys (<= candidates)
  // (the warp kernel's sizes need the longest incidence list, maxinc < 0:
  // not known yet -- the row-per-thread pass does without it)
  int hcap = 32, icap = 32, warps = 8;
  size_t smem = 0;
  auto setup_warp = [&]() -> int {
    if (maxinc < 0) GT_TRY(max_diff(ctx, A->inc_ptr, nrows, &maxinc));
    const int ncand_max = maxinc * NN;
    hcap = 32;
    icap = 32;
    while (hcap < ncand_max + ncand_max / 4) hcap <<= 1;
    while (icap < ncand_max) icap <<= 1;
    if (hcap > 8192) return set_error(ctx, GT_ERR_UNSUPPORTED, "a DOF touches too many cells for the sparsity kernel");
    warps = hcap >= 4096 ? 2 : (hcap >= 2048 ? 4 : 8);
    smem = (size_t)warps * (hcap + 2 * icap) * sizeof(int32_t);
    cudaFuncSetAttribute(k_pattern<NN, S, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_pattern<NN, S, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return GT_OK;
  };
  int32_t *rowcnt = nullptr, *dmax = nullptr, *slots = nullptr;
  uint8_t* small = nullptr;
  GT_TRY(dalloc(ctx, &rowcnt, nrows + 1));
  GT_TRY(dalloc(ctx, &dmax, 1));
  GT_TRY(dalloc(ctx, &slots, nrows * S));
  GT_TRY(dalloc(ctx, &small, nrows + 1));
  GT_TRY(dalloc(ctx, &A->rowptr, nrows + 1));
  // count pass: one thread per row where rows are short enough, else (or when
  // a row turned out longer than 32 incidences or columns) one warp per row
  bool rows_pass = NN <= 8 && S == kRowsS && ctx->pattern_rows;
  if (!rows_pass) GT_TRY(setup_warp());
  int32_t* dredo = nullptr;
  GT_TRY(dalloc(ctx, &dredo, 1));
  int32_t* dlast = nullptr;
  GT_TRY(dalloc(ctx, &dlast, kRowChunks));
  for (int attempt = 0; attempt < 2; attempt++) {
    const int grid = grid_for(nrows, warps);
    GT_CUDA(ctx, cudaMemsetAsync(dmax, 0, sizeof(int32_t), st));
    GT_CUDA(ctx, cudaMemsetAsync(dredo, 0, sizeof(int32_t), st));
    if (nrows > 0 && rows_pass) {
      // 16-bit column offsets when every column is within 2^15 of its row
      const bool c16 = sp->dof_spread >= 0 && sp->dof_spread < 32768;
      const size_t rsm = (size_t)128 * (kRowsMI * sizeof(int32_t) + kRowsS * (c16 ? sizeof(int16_t) : sizeof(int32_t)));
      if (c16)
        k_pattern_rows<NN, true><<<GT_KC(ctx, grid_for(nrows, 128)), 128, rsm, st>>>(
            A->inc_ptr, A->inc, sp->cell_ndofs, nrows, rowcnt, slots, small, dmax, dredo, bucket);
      else
        k_pattern_rows<NN, false><<<GT_KC(ctx, grid_for(nrows, 128)), 128, rsm, st>>>(
            A->inc_ptr, A->inc, sp->cell_ndofs, nrows, rowcnt, slots, small, dmax, dredo, bucket);
    } else if (nrows > 0) {
      k_pattern<NN, S, false><<<GT_KC(ctx, grid), warps * 32, smem, st>>>(A->inc_ptr, A->inc, sp->cell_ndofs, nrows,
                                                                          hcap, icap, rowcnt, nullptr, nullptr, slots,
                                                                          small, dmax, ctx->d_err);
    }
    GT_LAUNCH(ctx, "k_pattern<count>");
    GT_TRY(exclusive_scan_i64(ctx, rowcnt, A->rowptr, nrows));
    if (want_last) {
      GT_CUDA(ctx, cudaMemsetAsync(dlast, 0xff, sizeof(int32_t) * kRowChunks, st));
      if (nrows > 0)
        k_chunk_last<<<GT_KC(ctx, grid_for(nrows, 256)), 256, 0, st>>>(A->inc_ptr, A->inc, nrows, sp->nn, dlast);
      GT_LAUNCH(ctx, "k_chunk_last");
      GT_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scratch[16], dlast, sizeof(int32_t) * kRowChunks, cudaMemcpyDeviceToHost, st));
    }
    mark(ctx, "pattern_count");
    GT_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scratch[0], A->rowptr + nrows, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    GT_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scratch[1], dmax, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GT_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scratch[2], dredo, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    uint32_t bits = 0;
    GT_TRY(take_device_error(ctx, &bits));  // synchronises
    // bits of kernels on other streams (element checks) go back for the next take
    const uint32_t own = DEV_ERR_ROW_CAP | DEV_ERR_HASH_FULL;
    ctx->held_err |= bits & ~own;
    if (bits & own) return set_error(ctx, GT_ERR_INVALID, "sparsity: row capacity exceeded");
    int32_t redo = 0;
    memcpy(&redo, &ctx->h_scratch[2], sizeof(int32_t));
    if (!rows_pass || !redo) break;
    rows_pass = false;  // a row beyond 32 incidences or columns: count again, one warp per row
    if (bucket) {
      // the buckets kept only the first kIncBucket incidences of each row:
      // the whole incidence again, by count + fill (the stream is idle here)
      dfree(ctx, A->inc_ptr);
      dfree(ctx, A->inc);
      GT_TRY(build_incidence(ctx, sp, &A->inc_ptr, &A->inc, &A->ninc, false));
    }
    GT_TRY(setup_warp());
  }
  dfree(ctx, dredo);
  dfree(ctx, dlast);
  if (want_last) {
    memcpy(A->chunk_last, &ctx->h_scratch[16], sizeof(int32_t) * kRowChunks);
    A->chunk_last_ok = true;
  }
  A->bnnz = ctx->h_scratch[0];
  int32_t mr = 0;
  memcpy(&mr, &ctx->h_scratch[1], sizeof(int32_t));
  A->max_row = mr;
  GT_TRY(dalloc(ctx, &A->colind, A->bnnz));
  if (nrows > 0 && mr <= S) {
    // every row fit its slot: a plain coalesced copy
    k_copy_slots<S><<<GT_KC(ctx, grid_for(nrows * 4, 256)), 256, 0, st>>>(A->rowptr, slots, nrows, A->colind);
    GT_LAUNCH(ctx, "k_copy_slots");
  } else if (nrows > 0) {
    if (smem == 0) GT_TRY(setup_warp());
    const int grid = grid_for(nrows, warps);
    k_pattern<NN, S, true><<<GT_KC(ctx, grid), warps * 32, smem, st>>>(A->inc_ptr, A->inc, sp->cell_ndofs, nrows,
                                                                       hcap, icap, nullptr, A->rowptr, A->colind,
                                                                       slots, small, dmax, ctx->d_err);
    GT_LAUNCH(ctx, "k_pattern<fill>");
  }
  mark(ctx, "pattern_fill");
  dfree(ctx, rowcnt);
  dfree(ctx, dmax);
  dfree(ctx, slots);
  dfree(ctx, small);
  return GT_OK;
}

// incidence in one pass into row buckets (k_inc_place): row pointers from
// the counts, the lists themselves left to the count pass
static int build_incidence_bucket(Ctx* ctx, const Space* sp, int64_t** inc_ptr, int32_t** inc, int32_t** bucket) {
  cudaStream_t st = ctx->stream;
  const int64_t n = sp->mesh->ncells * sp->nn, nrows = sp->nfree_nodes;
  int32_t* cnt = nullptr;
  GT_TRY(dalloc(ctx, &cnt, nrows + 1));
  GT_TRY(dalloc(ctx, bucket, nrows > 0 ? nrows * kIncBucket : 1));
  GT_TRY(dalloc(ctx, inc_ptr, nrows + 1));
  GT_TRY(dalloc(ctx, inc, n > 0 ? n : 1));
  GT_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (nrows + 1), st));
  if (n > 0) k_inc_place<<<GT_KC(ctx, grid_for(n, 256)), 256, 0, st>>>(sp->cell_ndofs, n, cnt, *bucket);
  GT_LAUNCH(ctx, "k_inc_place");
  GT_TRY(exclusive_scan_i64(ctx, cnt, *inc_ptr, nrows));
  dfree(ctx, cnt);
  return GT_OK;
}

int build_pattern(Matrix* A, bool chunk_last) {
  const Space* sp = A->space;
  Ctx* ctx = sp->mesh->ctx;
  A->nbrows = sp->nfree_nodes;
  // P1/Q1 rows go through the row-per-thread count pass, whose incidence
  // comes in one pass through row buckets
  int32_t* bucket = nullptr;
  if ((sp->nn == 4 || sp->nn == 8) && ctx->pattern_rows) {
    GT_TRY(build_incidence_bucket(ctx, sp, &A->inc_ptr, &A->inc, &bucket));
    A->ninc = -1;
  } else {
    GT_TRY(build_incidence(ctx, sp, &A->inc_ptr, &A->inc, &A->ninc, false));
  }
  mark(ctx, "incidence");
  const int32_t maxinc = -1;  // computed by launch_pattern if the warp kernel runs
  int s = GT_OK;
  switch (sp->nn) {
    case 4: s = launch_pattern<4>(A, maxinc, bucket, chunk_last); break;
    case 8: s = launch_pattern<8>(A, maxinc, bucket, chunk_last); break;
    case 9: s = launch_pattern<9>(A, maxinc, nullptr, chunk_last); break;
    case 10: s = launch_pattern<10>(A, maxinc, nullptr, chunk_last); break;
    case 27: s = launch_pattern<27>(A, maxinc, nullptr, chunk_last); break;
    default: s = set_error(ctx, GT_ERR_UNSUPPORTED, "element not supported");
  }
  if (bucket) dfree(ctx, bucket);
  return s;
}

// ---------------------------------------------------------------------------
// 3. element matrices / vectors
// One CTA integrates CPB cells.  Phase 1: per (cell, quadrature point) the
// FP64 Jacobian J = sum_n x_n (x) grad m_n (src/accessors.jl:941-968), its
// inverse and determinant, dV = |det J| w (src/quadrature.jl:4-6) and the
// physical gradients J^-T grad_ref phi (src/accessors.jl:1365-1368), stored
// in shared memory in T.  Phase 2: per (cell, node pair n <= m) the BSxBS
// block of the element matrix, accumulated over quadrature points in T and
// written with its transpose.  Affine cells (TET4) compute J once per cell.
// ---------------------------------------------------------------------------
template <int D, int NLV, int NN, int NQ, int BS, int FORM, class T, int CPB, bool AFFINE>
__global__ void __launch_bounds__(128) k_elements(const double* __restrict__ coords, const int32_t* __restrict__ cell_nodes,
                                                  const double* __restrict__ coef, double nu,
                                                  const double* __restrict__ tab, TabLayout L, int64_t ncells,
                                                  T* __restrict__ Ke, double* __restrict__ be, const double* __restrict__ fsrc,
                                                  const double* __restrict__ scoef, int want_matrix, uint32_t* err) {
  constexpr int NLOC = NN * BS;
  constexpr int NQG = AFFINE ? 1 : NQ;  // quadrature points that carry gradients
  constexpr int NPAIR = NN * (NN + 1) / 2;
  __shared__ double s_x[CPB][NLV][D];
  __shared__ T s_g[CPB][NQG][NN][D];
  __shared__ T s_dv[CPB][NQ];
  __shared__ double s_tab[NQ * (1 + NLV * D + NN + NN * D)];
  const int tid = threadIdx.x;
  const int64_t c0 = (int64_t)blockIdx.x * CPB;
  // the tabulation proper (L.off_k entries; the P1 constants after it are not
  // staged) -- s_tab is sized for exactly this part
  static_assert(sizeof(s_tab) / sizeof(double) == NQ * (1 + NLV * D + NN + NN * D), "s_tab size");
  const int ntab = min(L.off_k, (int)(sizeof(s_tab) / sizeof(double)));
  for (int i = tid; i < ntab; i += blockDim.x) s_tab[i] = tab[i];
  for (int i = tid; i < CPB * NLV * D; i += blockDim.x) {
    int cl = i / (NLV * D), r = i - cl * NLV * D, n = r / D, d = r - n * D;
    int64_t c = c0 + cl;
    double v = 0.0;
    if (c < ncells) v = coords[(int64_t)cell_nodes[c * NLV + n] * D + d];
    s_x[cl][n][d] = v;
  }
  __syncthreads();
  const double* w = s_tab + L.off_w;
  const double* gg = s_tab + L.off_gg;
  const double* sv = s_tab + L.off_sv;
  const double* sg = s_tab + L.off_sg;
  // phase 1
  for (int item = tid; item < CPB * NQG; item += blockDim.x) {
    int cl = item / NQG, q = item - cl * NQG;
    double J[D][D];
#pragma unroll
    for (int i = 0; i < D; i++)
#pragma unroll
      for (int j = 0; j < D; j++) J[i][j] = 0.0;
#pragma unroll
    for (int n = 0; n < NLV; n++)
#pragma unroll
      for (int i = 0; i < D; i++)
#pragma unroll
        for (int j = 0; j < D; j++) J[i][j] = fma(s_x[cl][n][i], gg[(q * NLV + n) * D + j], J[i][j]);
    double inv[D][D], det;
    if (D == 2) {
      det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      double r = recip_nr2(det);
      inv[0][0] = J[1][1] * r; inv[0][1] = -J[0][1] * r;
      inv[1][0] = -J[1][0] * r; inv[1][1] = J[0][0] * r;
    } else {
      double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
      double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
      double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
      det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
      double r = recip_nr2(det);
      inv[0][0] = c00 * r; inv[1][0] = c01 * r; inv[2][0] = c02 * r;
      inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
      inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
      inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
      inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
      inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
      inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
    }
    if (c0 + cl < ncells && !(det != 0.0)) atomicOr(err, DEV_ERR_DEGENERATE);
    double adet = fabs(det);
    if (AFFINE) {
#pragma unroll
      for (int qq = 0; qq < NQ; qq++) s_dv[cl][qq] = (T)(adet * w[qq]);
    } else {
      s_dv[cl][q] = (T)(adet * w[q]);
    }
#pragma unroll 1
    for (int n = 0; n < NN; n++)
#pragma unroll
      for (int d = 0; d < D; d++) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < D; k++) s = fma(inv[k][d], sg[(q * NN + n) * D + k], s);
        s_g[cl][q][n][d] = (T)s;
      }
  }
  __syncthreads();
  // phase 2: element matrix blocks
  if (want_matrix) {
    const T lamf = (T)(nu / ((1.0 + nu) * (1.0 - 2.0 * nu))), muf = (T)(1.0 / (2.0 * (1.0 + nu)));
    for (int item = tid; item < CPB * NPAIR; item += blockDim.x) {
      int cl = item / NPAIR, p = item - cl * NPAIR;
      int64_t c = c0 + cl;
      if (c >= ncells) continue;
      // pair index -> (n, m) with n <= m
      int n = 0, rem = p;
      while (rem >= NN - n) { rem -= NN - n; n++; }
      int m = n + rem;
      T cf = (T)(coef ? coef[c] : 1.0);
      T blk[BS][BS];
      if (FORM == GT_ELASTICITY) {
        T A[D][D], sdot = 0;
#pragma unroll
        for (int a = 0; a < D; a++)
#pragma unroll
          for (int b = 0; b < D; b++) A[a][b] = 0;
#pragma unroll
        for (int q = 0; q < NQ; q++) {
          const int qg = AFFINE ? 0 : q;
          T dv = s_dv[cl][q];
          T gn[D], gm[D];
#pragma unroll
          for (int d = 0; d < D; d++) { gn[d] = s_g[cl][qg][n][d] * dv; gm[d] = s_g[cl][qg][m][d]; }
#pragma unroll
          for (int a = 0; a < D; a++) {
            sdot += gn[a] * gm[a];
#pragma unroll
            for (int b = 0; b < D; b++) A[a][b] += gn[a] * gm[b];
          }
        }
        T lam = cf * lamf, mu = cf * muf;
#pragma unroll
        for (int a = 0; a < BS; a++)
#pragma unroll
          for (int b = 0; b < BS; b++) blk[a][b] = lam * A[a][b] + mu * A[b][a] + (a == b ? mu * sdot : (T)0);
      } else {
        T acc = 0;
        if (FORM == GT_LAPLACE) {
          if (AFFINE) {
            T dvs = 0, dot = 0;
#pragma unroll
            for (int q = 0; q < NQ; q++) dvs += s_dv[cl][q];
#pragma unroll
            for (int d = 0; d < D; d++) dot += s_g[cl][0][n][d] * s_g[cl][0][m][d];
            acc = dot * dvs;
          } else {
#pragma unroll
            for (int q = 0; q < NQ; q++) {
              T dot = 0;
#pragma unroll
              for (int d = 0; d < D; d++) dot += s_g[cl][q][n][d] * s_g[cl][q][m][d];
              acc += dot * s_dv[cl][q];
            }
          }
        } else {
#pragma unroll
          for (int q = 0; q < NQ; q++) acc += (T)(sv[q * NN + n] * sv[q * NN + m]) * s_dv[cl][q];
        }
        acc *= cf;
#pragma unroll
        for (int a = 0; a < BS; a++)
#pragma unroll
          for (int b = 0; b < BS; b++) blk[a][b] = a == b ? acc : (T)0;
      }
      T* K = Ke + c * (NLOC * NLOC);
#pragma unroll
      for (int a = 0; a < BS; a++)
#pragma unroll
        for (int b = 0; b < BS; b++) {
          K[(n * BS + a) * NLOC + m * BS + b] = blk[a][b];
          K[(m * BS + b) * NLOC + n * BS + a] = blk[a][b];
        }
    }
  }
  // element vector: int coef f . v dOmega
  if (be) {
    for (int item = tid; item < CPB * NN; item += blockDim.x) {
      int cl = item / NN, n = item - cl * NN;
      int64_t c = c0 + cl;
      if (c >= ncells) continue;
      double cf = scoef ? scoef[c] : 1.0;
      double s = 0.0;
      for (int q = 0; q < NQ; q++) s += sv[q * NN + n] * (double)s_dv[cl][q];
#pragma unroll
      for (int k = 0; k < BS; k++) be[c * NLOC + n * BS + k] = cf * fsrc[k] * s;
    }
  }
}

template <int D, int NLV, int NN, int NQ, int BS, int FORM, class T, int CPB, bool AFFINE>
static int launch_elements(const Space* sp, const double* coef, double nu, const double* tab, const TabLayout& L, T* Ke,
                           double* be, const double* f, const double* scoef, int want_matrix) {
  Ctx* ctx = sp->mesh->ctx;
  int64_t nc = sp->mesh->ncells;
  int64_t grid = (nc + CPB - 1) / CPB;
  k_elements<D, NLV, NN, NQ, BS, FORM, T, CPB, AFFINE><<<GT_KC(ctx, (unsigned)grid), 128, 0, ctx->stream>>>(
      sp->mesh->coords, sp->mesh->cell_nodes, coef, nu, tab, L, nc, Ke, be, f, scoef, want_matrix, ctx->d_err);
  GT_LAUNCH(ctx, "k_elements");
  return GT_OK;
}

template <int D, int NLV, int NN, int NQ, int CPB, bool AFFINE, class T>
static int dispatch_form(const Space* sp, int form, const double* coef, double nu, const double* tab, const TabLayout& L,
                         T* Ke, double* be, const double* f, const double* scoef, int want_matrix) {
  int bs = sp->ncomp;
  if (bs == 1) {
    if (form == GT_LAPLACE)
      return launch_elements<D, NLV, NN, NQ, 1, GT_LAPLACE, T, CPB, AFFINE>(sp, coef, nu, tab, L, Ke, be, f, scoef, want_matrix);
    if (form == GT_MASS)
      return launch_elements<D, NLV, NN, NQ, 1, GT_MASS, T, CPB, AFFINE>(sp, coef, nu, tab, L, Ke, be, f, scoef, want_matrix);
  } else {
    if (form == GT_LAPLACE)
      return launch_elements<D, NLV, NN, NQ, D, GT_LAPLACE, T, CPB, AFFINE>(sp, coef, nu, tab, L, Ke, be, f, scoef, want_matrix);
    if (form == GT_MASS)
      return launch_elements<D, NLV, NN, NQ, D, GT_MASS, T, CPB, AFFINE>(sp, coef, nu, tab, L, Ke, be, f, scoef, want_matrix);
    if (form == GT_ELASTICITY)
      return launch_elements<D, NLV, NN, NQ, D, GT_ELASTICITY, T, CPB, AFFINE>(sp, coef, nu, tab, L, Ke, be, f,
                                                                               scoef, want_matrix);
  }
  return set_error(ctx_of(sp), GT_ERR_UNSUPPORTED, "weak form not supported on this space");
}


// P1 tetrahedra, scalar Laplacian / mass: one thread per cell.  The map is
// affine, so J = [x1-x0, x2-x0, x3-x0] is constant over the cell and the
// physical gradients are the columns c_j of the cofactor matrix of J divided
// by det J (J^-T = cof(J) / det J), with c_0 = -(c_1 + c_2 + c_3).  Then
//   Laplacian  K_nm = coef * (sum_q w_q) / |det J| * (c_n . c_m)
//   mass       K_nm = coef * |det J| * sum_q w_q phi_n(q) phi_m(q)
// -- the quadrature sums of the reference loop (src/compiler.jl:1865-1917
// with dV = |det J| w, src/quadrature.jl:4-6) with the constant factors
// taken out: one FP64 division and ~80 FP64 operations per cell.  J, its
// cofactors and det stay FP64 in every precision; in FP32 mode the cofactor
// columns are rounded to FP32 for the entries.
// the quadrature sums of the P1 reference cell, once per assembly:
// k[0] = sum_q w_q, k[1..4] = sum_q w_q phi_n(q), k[5..20] = sum_q w_q phi_n phi_m,
// k[21] = 1 when k[1..4] are bitwise equal (a symmetric rule), else 0
__global__ void k_p1_consts(const double* __restrict__ tab, TabLayout L, double* __restrict__ k) {
  const int t = threadIdx.x;
  double s = 0.0;
  if (t == 0) {
    for (int q = 0; q < 4; q++) s += tab[L.off_w + q];
  } else if (t < 5) {
    for (int q = 0; q < 4; q++) s += tab[L.off_w + q] * tab[L.off_sv + q * 4 + (t - 1)];
  } else if (t < 21) {
    const int n = (t - 5) >> 2, m = (t - 5) & 3;
    for (int q = 0; q < 4; q++) s += tab[L.off_w + q] * tab[L.off_sv + q * 4 + n] * tab[L.off_sv + q * 4 + m];
  }
  if (t < 21) k[t] = s;
  long long b[4];
#pragma unroll
  for (int n = 0; n < 4; n++) b[n] = __double_as_longlong(__shfl_sync(0xffffffffu, s, n + 1));
  if (t == 21) k[t] = (b[0] == b[1] && b[0] == b[2] && b[0] == b[3]) ? 1.0 : 0.0;
  // the sums as FP32 pairs for the double-float kernel (from k[24] on, as
  // floats): [0,1] sum w, [2..9] the four load sums, [10..29] the ten
  // upper-triangle mass sums in the packed order
  float* kf = reinterpret_cast<float*>(k + 24);
  if (t < 5) {
    const dfl v = df_from_double(s);
    kf[2 * t] = v.hi;
    kf[2 * t + 1] = v.lo;
  } else if (t < 21) {
    const int n = (t - 5) >> 2, m = (t - 5) & 3;
    if (n <= m) {
      const int e = n * 4 - ((n * (n - 1)) >> 1) + (m - n);
      const dfl v = df_from_double(s);
      kf[10 + 2 * e] = v.hi;
      kf[11 + 2 * e] = v.lo;
    }
  }
}

template <int FORM, class T>
__global__ void __launch_bounds__(256) k_elements_p1(const double* __restrict__ coords,
                                                     const int32_t* __restrict__ cell_nodes,
                                                     const double* __restrict__ coef,
                                                     const double* __restrict__ consts, int64_t c_begin,
                                                     int64_t ncells, T* __restrict__ Ke, double* __restrict__ be,
                                                     const double* __restrict__ fsrc,
                                                     const double* __restrict__ scoef, int want_matrix, uint32_t* err) {
  const double* s_load = consts + 1;
  const double* s_mass = consts + 5;
  const double s_wsum = __ldg(consts);
  // uniform over the launch: one load entry for all four nodes, and the
  // source value without a cell coefficient (1 * f is f)
  const bool load_equal = __double_as_longlong(__ldg(consts + 21)) != 0;
  const double f0 = fsrc ? __ldg(fsrc) : 0.0;
  // grid-stride over the cells [c_begin, ncells) (one thread per cell)
  for (int64_t c = c_begin + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells;
       c += (int64_t)gridDim.x * blockDim.x) {
    int4 nd = *reinterpret_cast<const int4*>(cell_nodes + 4 * c);
    const double* p0 = coords + 3 * (int64_t)nd.x;
    const double* p1 = coords + 3 * (int64_t)nd.y;
    const double* p2 = coords + 3 * (int64_t)nd.z;
    const double* p3 = coords + 3 * (int64_t)nd.w;
    double x0 = p0[0], y0 = p0[1], z0 = p0[2];
    // J columns
    double a0 = p1[0] - x0, a1 = p1[1] - y0, a2 = p1[2] - z0;
    double b0 = p2[0] - x0, b1 = p2[1] - y0, b2 = p2[2] - z0;
    double d0 = p3[0] - x0, d1 = p3[1] - y0, d2 = p3[2] - z0;
    // J = [[a0 b0 d0],[a1 b1 d1],[a2 b2 d2]]; cofactor columns C[:,j]
    double c10 = b1 * d2 - b2 * d1, c11 = b2 * d0 - b0 * d2, c12 = b0 * d1 - b1 * d0;  // column 0 (row of J^-1 #0)
    double c20 = d1 * a2 - d2 * a1, c21 = d2 * a0 - d0 * a2, c22 = d0 * a1 - d1 * a0;  // column 1
    double c30 = a1 * b2 - a2 * b1, c31 = a2 * b0 - a0 * b2, c32 = a0 * b1 - a1 * b0;  // column 2
    double det = a0 * c10 + a1 * c11 + a2 * c12;
    // det == +-0 tested on its bits: integer instructions, not an FP64 compare
    if ((__double_as_longlong(det) << 1) == 0) atomicOr(err, DEV_ERR_DEGENERATE);
    double adet = fabs(det);
    double cf = coef ? coef[c] : 1.0;
    if (want_matrix) {
      T k[10];
      if (FORM == GT_LAPLACE) {
        // the six entries among vertices 1..3 from the cofactor columns; the
        // entries of vertex 0 follow from c_0 = -(c_1 + c_2 + c_3), i.e. from
        // the zero row sums of the Laplacian (8 additions instead of 4 dot
        // products: the kernel is bound by the FP64 issue rate)
        T g[3][3];
        g[0][0] = (T)c10; g[0][1] = (T)c11; g[0][2] = (T)c12;
        g[1][0] = (T)c20; g[1][1] = (T)c21; g[1][2] = (T)c22;
        g[2][0] = (T)c30; g[2][1] = (T)c31; g[2][2] = (T)c32;
        T s = (T)(cf * s_wsum * recip_nr2(adet));
        T k11 = s * (g[0][0] * g[0][0] + g[0][1] * g[0][1] + g[0][2] * g[0][2]);
        T k12 = s * (g[0][0] * g[1][0] + g[0][1] * g[1][1] + g[0][2] * g[1][2]);
        T k13 = s * (g[0][0] * g[2][0] + g[0][1] * g[2][1] + g[0][2] * g[2][2]);
        T k22 = s * (g[1][0] * g[1][0] + g[1][1] * g[1][1] + g[1][2] * g[1][2]);
        T k23 = s * (g[1][0] * g[2][0] + g[1][1] * g[2][1] + g[1][2] * g[2][2]);
        T k33 = s * (g[2][0] * g[2][0] + g[2][1] * g[2][1] + g[2][2] * g[2][2]);
        T k01 = -(k11 + k12 + k13), k02 = -(k12 + k22 + k23), k03 = -(k13 + k23 + k33);
        T k00 = -(k01 + k02 + k03);
        k[0] = k00; k[1] = k01; k[2] = k02; k[3] = k03;
        k[4] = k11; k[5] = k12; k[6] = k13;
        k[7] = k22; k[8] = k23;
        k[9] = k33;
      } else {
        T s = (T)(cf * adet);
        int e = 0;
  #pragma unroll
        for (int n = 0; n < 4; n++)
  #pragma unroll
          for (int m = n; m < 4; m++) k[e++] = s * (T)__ldg(s_mass + n * 4 + m);
      }
      // packed upper triangle (the matrix is symmetric): 10 entries per cell
      T* K = Ke + 10 * c;
  #pragma unroll
      for (int e = 0; e < 10; e++) K[e] = k[e];
    }
    if (be) {
      const double sc = (scoef ? scoef[c] * f0 : f0) * adet;
      if (load_equal) {
        const double v = sc * __ldg(s_load);
        double2* b2 = reinterpret_cast<double2*>(be + 4 * c);  // 32-byte records of a pool block
        b2[0] = make_double2(v, v);
        b2[1] = make_double2(v, v);
      } else {
  #pragma unroll
        for (int n = 0; n < 4; n++) be[4 * c + n] = sc * __ldg(s_load + n);
      }
    }
  }
}

// The FP64-valued P1 kernel in double-float arithmetic (gt_dfloat.cuh):
// the same formulas and summation order as k_elements_p1<FORM, double>, with
// J's nine differences taken in FP64 (x_i - x_0 loses nothing there) and
// everything after them -- cofactors, det J, its reciprocal, the entries,
// the load vector -- in pairs of FP32 numbers (48 significant bits) on the
// FP32 pipes; the matrix entries leave as pairs (the scatter rounds each CSR
// value to FP64 once).  About 9 FP64 instructions per cell instead of ~75,
// so the kernel is no longer bound by GB300's FP64 rate.  Its sums are the
// sloppy double-float sum (error ~2^-47 of the terms, which are of the size
// of the element matrix's entries): the values agree with the FP64 kernel's
// (and the FP64 oracle's) to a few units of 2^-47 relative to the largest
// entry, far inside the 1e-12 parity tolerance.
template <int FORM>
__global__ void __launch_bounds__(256) k_elements_p1_df(const double* __restrict__ coords,
                                                        const int32_t* __restrict__ cell_nodes,
                                                        const double* __restrict__ coef,
                                                        const double* __restrict__ consts, int64_t c_begin,
                                                        int64_t ncells, double* __restrict__ Ke,
                                                        double* __restrict__ be, const double* __restrict__ fsrc,
                                                        const double* __restrict__ scoef, int want_matrix,
                                                        uint32_t* err) {
  // the reference-cell sums as FP32 pairs, split once by k_p1_consts
  const float* kf = reinterpret_cast<const float*>(consts + 24);
  const dfl wsum = {__ldg(kf), __ldg(kf + 1)};
  const bool load_equal = __double_as_longlong(__ldg(consts + 21)) != 0;
  dfl sload[4], smass[10];
#pragma unroll
  for (int n = 0; n < 4; n++) sload[n] = {__ldg(kf + 2 + 2 * n), __ldg(kf + 3 + 2 * n)};
  if (FORM == GT_MASS) {
#pragma unroll
    for (int e = 0; e < 10; e++) smass[e] = {__ldg(kf + 10 + 2 * e), __ldg(kf + 11 + 2 * e)};
  }
  const dfl one = {1.0f, 0.0f};
  for (int64_t c = c_begin + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells;
       c += (int64_t)gridDim.x * blockDim.x) {
    int4 nd = *reinterpret_cast<const int4*>(cell_nodes + 4 * c);
    const double* p0 = coords + 3 * (int64_t)nd.x;
    const double* p1 = coords + 3 * (int64_t)nd.y;
    const double* p2 = coords + 3 * (int64_t)nd.z;
    const double* p3 = coords + 3 * (int64_t)nd.w;
    const double x0 = p0[0], y0 = p0[1], z0 = p0[2];
    // J columns a, b, d (FP64 differences), then double-float
    const dfl a[3] = {df_from_double(p1[0] - x0), df_from_double(p1[1] - y0), df_from_double(p1[2] - z0)};
    const dfl b[3] = {df_from_double(p2[0] - x0), df_from_double(p2[1] - y0), df_from_double(p2[2] - z0)};
    const dfl d[3] = {df_from_double(p3[0] - x0), df_from_double(p3[1] - y0), df_from_double(p3[2] - z0)};
    // cofactor columns c_1, c_2, c_3 (the physical gradients times det J)
    const dfl g1[3] = {df_mul_sub_s(b[1], d[2], b[2], d[1]), df_mul_sub_s(b[2], d[0], b[0], d[2]),
                       df_mul_sub_s(b[0], d[1], b[1], d[0])};
    const dfl det = df_dot3_s(a, g1);
    if (det.hi == 0.0f) atomicOr(err, DEV_ERR_DEGENERATE);
    const dfl adet = df_abs(det);
    const dfl cf = coef ? df_from_double(coef[c]) : one;
    if (want_matrix) {
      dfl k[10];
      if (FORM == GT_LAPLACE) {
        const dfl g2[3] = {df_mul_sub_s(d[1], a[2], d[2], a[1]), df_mul_sub_s(d[2], a[0], d[0], a[2]),
                           df_mul_sub_s(d[0], a[1], d[1], a[0])};
        const dfl g3[3] = {df_mul_sub_s(a[1], b[2], a[2], b[1]), df_mul_sub_s(a[2], b[0], a[0], b[2]),
                           df_mul_sub_s(a[0], b[1], a[1], b[0])};
        const dfl s = df_mul(df_mul(cf, wsum), df_recip_s(adet));
        const dfl k11 = df_mul(s, df_dot3_s(g1, g1)), k12 = df_mul(s, df_dot3_s(g1, g2)), k13 = df_mul(s, df_dot3_s(g1, g3));
        const dfl k22 = df_mul(s, df_dot3_s(g2, g2)), k23 = df_mul(s, df_dot3_s(g2, g3));
        const dfl k33 = df_mul(s, df_dot3_s(g3, g3));
        // vertex 0 from the zero row sums, as in the FP64 kernel
        const dfl k01 = df_neg(df_add_sloppy(df_add_sloppy(k11, k12), k13));
        const dfl k02 = df_neg(df_add_sloppy(df_add_sloppy(k12, k22), k23));
        const dfl k03 = df_neg(df_add_sloppy(df_add_sloppy(k13, k23), k33));
        const dfl k00 = df_neg(df_add_sloppy(df_add_sloppy(k01, k02), k03));
        k[0] = k00; k[1] = k01; k[2] = k02; k[3] = k03;
        k[4] = k11; k[5] = k12; k[6] = k13;
        k[7] = k22; k[8] = k23;
        k[9] = k33;
      } else {
        const dfl s = df_mul(cf, adet);
#pragma unroll
        for (int e = 0; e < 10; e++) k[e] = df_mul(s, smass[e]);
      }
      // the entries stay double-float pairs: the scatter sums them as such
      // and rounds each CSR value to FP64 once
      float2* K = reinterpret_cast<float2*>(Ke + 10 * c);
#pragma unroll
      for (int e = 0; e < 10; e++) K[e] = make_float2(k[e].hi, k[e].lo);
    }
    if (be) {
      const dfl f0 = fsrc ? df_from_double(__ldg(fsrc)) : dfl{0.0f, 0.0f};  // only with a load vector
      const dfl sc = df_mul(scoef ? df_mul(df_from_double(scoef[c]), f0) : f0, adet);
      if (load_equal) {
        const double v = df_to_double(df_mul(sc, sload[0]));
        double2* b2 = reinterpret_cast<double2*>(be + 4 * c);  // 32-byte records of a pool block
        b2[0] = make_double2(v, v);
        b2[1] = make_double2(v, v);
      } else {
#pragma unroll
        for (int n = 0; n < 4; n++) be[4 * c + n] = df_to_double(df_mul(sc, sload[n]));
      }
    }
  }
}

// element kernels per cell type / order; returns GT_OK or an error
template <class T>
static int elements_T(const Space* sp, int form, const double* coef, double nu, const double* tab, const TabLayout& L,
                      T* Ke, double* be, const double* f, const double* scoef, int want_matrix,
                      ElemChunks* chunks = nullptr) {
  if (chunks && !(sp->mesh->ctype == GT_TET4 && sp->order == 1 && sp->ncomp == 1)) chunks->n = 0;
  int ct = sp->mesh->ctype, o = sp->order;
  if (ct == GT_TET4 && o == 1 && sp->ncomp == 1 && (form == GT_LAPLACE || form == GT_MASS)) {
    Ctx* ctx = ctx_of(sp);
    int64_t nc = sp->mesh->ncells;
    double* consts = const_cast<double*>(tab) + L.off_k;  // inside the tabulation buffer: no allocation
    k_p1_consts<<<GT_KC(ctx, 1), 32, 0, ctx->stream>>>(tab, L, consts);
    // one launch, or one per cell chunk with the chunk's event behind it
    const int nch = chunks ? chunks->n : 1;
    for (int i = 0; i < nch; i++) {
      const int64_t c0 = nc * i / nch, c1 = nc * (i + 1) / nch;
      const int grid = grid_for(c1 - c0 > 0 ? c1 - c0 : 1, 256);
      bool df = false;
      if constexpr (std::is_same<T, double>::value) df = ctx->p1_dfloat;
      if (df) {
        if constexpr (std::is_same<T, double>::value) {
          if (form == GT_LAPLACE)
            k_elements_p1_df<GT_LAPLACE><<<GT_KC(ctx, grid), 256, 0, ctx->stream>>>(
                sp->mesh->coords, sp->mesh->cell_nodes, coef, consts, c0, c1, Ke, be, f, scoef, want_matrix, ctx->d_err);
          else
            k_elements_p1_df<GT_MASS><<<GT_KC(ctx, grid), 256, 0, ctx->stream>>>(
                sp->mesh->coords, sp->mesh->cell_nodes, coef, consts, c0, c1, Ke, be, f, scoef, want_matrix, ctx->d_err);
        }
      } else if (form == GT_LAPLACE) {
        k_elements_p1<GT_LAPLACE, T><<<GT_KC(ctx, grid), 256, 0, ctx->stream>>>(
            sp->mesh->coords, sp->mesh->cell_nodes, coef, consts, c0, c1, Ke, be, f, scoef, want_matrix, ctx->d_err);
      } else {
        k_elements_p1<GT_MASS, T><<<GT_KC(ctx, grid), 256, 0, ctx->stream>>>(
            sp->mesh->coords, sp->mesh->cell_nodes, coef, consts, c0, c1, Ke, be, f, scoef, want_matrix, ctx->d_err);
      }
      GT_LAUNCH(ctx, "k_elements_p1");
      if (chunks) {
        chunks->end[i] = c1;
        GT_CUDA(ctx, cudaEventRecord(chunks->ev[i], ctx->stream));
      }
    }
    return GT_OK;
  }
  // P2 tets: the map is affine but the shape gradients vary over the cell, so
  // they are kept per quadrature point (the non-affine form of the kernel)
  if (ct == GT_TET4 && o == 2) return dispatch_form<3, 4, 10, 11, 8, false, T>(sp, form, coef, nu, tab, L, Ke, be, f, scoef, want_matrix);
  if (ct == GT_TET4) return dispatch_form<3, 4, 4, 4, 128, true, T>(sp, form, coef, nu, tab, L, Ke, be, f, scoef, want_matrix);
  if (ct == GT_QUAD4 && o == 1) return dispatch_form<2, 4, 4, 4, 32, false, T>(sp, form, coef, nu, tab, L, Ke, be, f, scoef, want_matrix);
  if (ct == GT_QUAD4 && o == 2) return dispatch_form<2, 4, 9, 9, 8, false, T>(sp, form, coef, nu, tab, L, Ke, be, f, scoef, want_matrix);
  if (ct == GT_HEX8 && o == 1) return dispatch_form<3, 8, 8, 8, 8, false, T>(sp, form, coef, nu, tab, L, Ke, be, f, scoef, want_matrix);
  if (ct == GT_HEX8 && o == 2) return dispatch_form<3, 8, 27, 27, 1, false, T>(sp, form, coef, nu, tab, L, Ke, be, f, scoef, want_matrix);
  return set_error(ctx_of(sp), GT_ERR_UNSUPPORTED, "element not supported");
}

int compute_elements(const Space* sp, int form, const double* d_coef, double nu, int precision, const double* f,
                     const double* d_scoef, void* Ke, double* be, int want_matrix, double** keep_tab,
                     ElemChunks* chunks) {
  Ctx* ctx = ctx_of(sp);
  if (form != GT_LAPLACE && form != GT_MASS && form != GT_ELASTICITY)
    return set_error(ctx, GT_ERR_UNSUPPORTED, "weak form not supported (Laplacian, mass, linear elasticity only)");
  if (form == GT_ELASTICITY && sp->ncomp != sp->mesh->D)
    return set_error(ctx, GT_ERR_UNSUPPORTED, "linear elasticity needs a vector space (tensor_size = (D,))");
  double* tab = nullptr;
  TabLayout L;
  GT_TRY(get_tab(ctx, sp->mesh->ctype, sp->order, &tab, &L));
  int s;
  if (precision == GT_FP32)
    s = elements_T<float>(sp, form, d_coef, nu, tab, L, (float*)Ke, be, f, d_scoef, want_matrix, chunks);
  else
    s = elements_T<double>(sp, form, d_coef, nu, tab, L, (double*)Ke, be, f, d_scoef, want_matrix, chunks);
  if (keep_tab) *keep_tab = tab;
  else dfree(ctx, tab);
  return s;
}

// ---------------------------------------------------------------------------
// Integrals over the cells: GT.assemble_scalar (src/problems.jl:172-190) for
// the fixed integrands the reference's tests integrate -- 1, a polynomial,
// the discrete field, its square, and the squared L2 / H1-seminorm errors
// against a polynomial (test/integration_tests.jl:68-77, the patch tests of
// test/assembly_tests.jl:43-118).  Same quadrature as the assembly, dV =
// |det J| w (src/quadrature.jl:4-6), grad u = J^-T grad u^ (src/accessors.jl:
// 1365-1373).  One thread per cell; per-cell values summed in a fixed order.
// ---------------------------------------------------------------------------
// p(x) with coefficients of 1, x, y, z, x^2, y^2, z^2, xy, xz, yz, and its gradient
__device__ __forceinline__ double poly_eval(const double* c, const double* x, double* g) {
  const double X = x[0], Y = x[1], Z = x[2];
  g[0] = c[1] + 2.0 * c[4] * X + c[7] * Y + c[8] * Z;
  g[1] = c[2] + 2.0 * c[5] * Y + c[7] * X + c[9] * Z;
  g[2] = c[3] + 2.0 * c[6] * Z + c[8] * X + c[9] * Y;
  return c[0] + c[1] * X + c[2] * Y + c[3] * Z + c[4] * X * X + c[5] * Y * Y + c[6] * Z * Z + c[7] * X * Y +
         c[8] * X * Z + c[9] * Y * Z;
}

constexpr int kPolyCoefs = 10;

template <int D, int NLV, int NN>
__global__ void __launch_bounds__(128) k_integrate(const double* __restrict__ coords, const int32_t* __restrict__ cell_nodes,
                                                   const int32_t* __restrict__ cnd, const double* __restrict__ tab,
                                                   TabLayout L, int64_t ncells, int ncomp, int kind,
                                                   const double* __restrict__ uf, const double* __restrict__ ud,
                                                   const double* __restrict__ poly, double* __restrict__ cell_val) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  double X[NLV][3];
#pragma unroll
  for (int v = 0; v < NLV; v++) {
    const int64_t nd = cell_nodes[c * NLV + v];
#pragma unroll
    for (int d = 0; d < 3; d++) X[v][d] = d < D ? coords[nd * D + d] : 0.0;
  }
  const bool want_u = kind >= GT_INT_FIELD;
  int32_t dof[NN];
#pragma unroll
  for (int n = 0; n < NN; n++) dof[n] = want_u ? cnd[c * NN + n] : 0;
  double acc = 0.0;
  for (int q = 0; q < L.nq; q++) {
    double J[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, x[3] = {0, 0, 0};
#pragma unroll
    for (int i = 0; i < D; i++)
#pragma unroll
      for (int j = 0; j < D; j++) J[i][j] = 0.0;
#pragma unroll
    for (int v = 0; v < NLV; v++) {
      const double gv = tab[L.off_gv + q * NLV + v];
#pragma unroll
      for (int i = 0; i < D; i++) {
        x[i] += X[v][i] * gv;
#pragma unroll
        for (int j = 0; j < D; j++) J[i][j] += X[v][i] * tab[L.off_gg + (q * NLV + v) * D + j];
      }
    }
    double det, inv[3][3];
    if (D == 2) {
      det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      const double r = 1.0 / det;
      inv[0][0] = J[1][1] * r; inv[0][1] = -J[0][1] * r; inv[1][0] = -J[1][0] * r; inv[1][1] = J[0][0] * r;
    } else {
      const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1], c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2],
                   c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
      det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
      const double r = 1.0 / det;
      inv[0][0] = c00 * r; inv[1][0] = c01 * r; inv[2][0] = c02 * r;
      inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
      inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
      inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
      inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
      inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
      inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
    }
    const double dv = fabs(det) * tab[L.off_w + q];
    if (kind == GT_INT_VOLUME) {
      acc += dv;
      continue;
    }
    double pg[3];
    if (kind == GT_INT_POLY) {
      acc += dv * poly_eval(poly, x, pg);
      continue;
    }
    double term = 0.0;
    for (int k = 0; k < ncomp; k++) {
      double u = 0.0, gr[3] = {0, 0, 0};
#pragma unroll
      for (int n = 0; n < NN; n++) {
        const int32_t d = dof[n];
        const double val = d > 0 ? uf[(int64_t)(d - 1) * ncomp + k] : (ud ? ud[(int64_t)(-d - 1) * ncomp + k] : 0.0);
        u += val * tab[L.off_sv + q * NN + n];
        if (kind == GT_INT_H1_ERROR2)
#pragma unroll
          for (int j = 0; j < D; j++) gr[j] += val * tab[L.off_sg + (q * NN + n) * D + j];
      }
      if (kind == GT_INT_FIELD) {
        term += u;
      } else if (kind == GT_INT_L2_NORM2) {
        term += u * u;
      } else {
        const double p = poly_eval(poly + k * kPolyCoefs, x, pg);
        if (kind == GT_INT_L2_ERROR2) {
          term += (u - p) * (u - p);
        } else {
          // physical gradient: sum_j inv[j][i] * ref gradient j  (J^-T)
#pragma unroll
          for (int i = 0; i < D; i++) {
            double g = 0.0;
#pragma unroll
            for (int j = 0; j < D; j++) g += inv[j][i] * gr[j];
            term += (g - pg[i]) * (g - pg[i]);
          }
        }
      }
    }
    acc += dv * term;
  }
  cell_val[c] = acc;
}

// fixed-order sums of 2048 consecutive values per CTA (strided per thread,
// then a tree); the host adds the CTA sums in order
__global__ void k_sum_fixed(const double* __restrict__ v, int64_t n, double* __restrict__ part) {
  __shared__ double t[256];
  const int64_t b0 = (int64_t)blockIdx.x * 2048;
  double s = 0.0;
  for (int k = 0; k < 8; k++) {
    const int64_t i = b0 + (int64_t)k * 256 + threadIdx.x;
    if (i < n) s += v[i];
  }
  t[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o; o >>= 1) {
    if ((int)threadIdx.x < o) t[threadIdx.x] += t[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = t[0];
}

template <int D, int NLV, int NN>
static void launch_integrate(const Space* sp, const double* tab, const TabLayout& L, int kind, const double* uf,
                             const double* ud, const double* poly, double* cell_val) {
  Ctx* ctx = ctx_of(sp);
  const int64_t nc = sp->mesh->ncells;
  k_integrate<D, NLV, NN><<<GT_KC(ctx, grid_for(nc, 128)), 128, 0, ctx->stream>>>(
      sp->mesh->coords, sp->mesh->cell_nodes, sp->cell_ndofs, tab, L, nc, sp->ncomp, kind, uf, ud, poly, cell_val);
}

static int integrate(const Space* sp, int kind, const double* uf, const double* ud, const double* poly, double* out) {
  Ctx* ctx = ctx_of(sp);
  const int ct = sp->mesh->ctype, o = sp->order;
  const int64_t nc = sp->mesh->ncells;
  *out = 0.0;
  if (nc == 0) return GT_OK;
  mesh_wait_coords(sp->mesh);
  double* tab = nullptr;
  TabLayout L;
  GT_TRY(get_tab(ctx, ct, o, &tab, &L));
  double *cv = nullptr, *part = nullptr;
  const int64_t nb = (nc + 2047) / 2048;
  int s = dalloc(ctx, &cv, nc);
  if (s == GT_OK) s = dalloc(ctx, &part, nb);
  if (s == GT_OK) {
    if (ct == GT_TET4 && o == 2) launch_integrate<3, 4, 10>(sp, tab, L, kind, uf, ud, poly, cv);
    else if (ct == GT_TET4) launch_integrate<3, 4, 4>(sp, tab, L, kind, uf, ud, poly, cv);
    else if (ct == GT_QUAD4 && o == 1) launch_integrate<2, 4, 4>(sp, tab, L, kind, uf, ud, poly, cv);
    else if (ct == GT_QUAD4) launch_integrate<2, 4, 9>(sp, tab, L, kind, uf, ud, poly, cv);
    else if (o == 1) launch_integrate<3, 8, 8>(sp, tab, L, kind, uf, ud, poly, cv);
    else launch_integrate<3, 8, 27>(sp, tab, L, kind, uf, ud, poly, cv);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) s = check_cuda(ctx, e, "k_integrate");
  }
  if (s == GT_OK) {
    k_sum_fixed<<<GT_KC(ctx, (unsigned)nb), 256, 0, ctx->stream>>>(cv, nc, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) s = check_cuda(ctx, e, "k_sum_fixed");
  }
  std::vector<double> h((size_t)nb);
  if (s == GT_OK) s = copy_out(ctx, h.data(), part, nb);
  if (s == GT_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) s = check_cuda(ctx, e, "integrate");
  }
  if (s == GT_OK) {
    double t = 0.0;
    for (int64_t i = 0; i < nb; i++) t += h[(size_t)i];
    *out = t;
  }
  dfree(ctx, tab);
  dfree(ctx, cv);
  dfree(ctx, part);
  return s;
}

// Number of doubles of the tabulation buffer of a space's reference cell.
int tabulation_doubles(const Space* sp) { return tab_layout(sp->mesh->ctype, sp->order).total; }

// Element matrices with a caller-provided tabulation buffer (no allocation).
int compute_elements_with_tab(const Space* sp, int form, const double* d_coef, double nu, int precision, double* tab,
                              void* Ke) {
  Ctx* ctx = ctx_of(sp);
  mesh_wait_coords(sp->mesh);
  if (form != GT_LAPLACE && form != GT_MASS && form != GT_ELASTICITY)
    return set_error(ctx, GT_ERR_UNSUPPORTED, "weak form not supported (Laplacian, mass, linear elasticity only)");
  if (form == GT_ELASTICITY && sp->ncomp != sp->mesh->D)
    return set_error(ctx, GT_ERR_UNSUPPORTED, "linear elasticity needs a vector space (tensor_size = (D,))");
  TabLayout L = tab_layout(sp->mesh->ctype, sp->order);
  k_tabulate<<<GT_KC(ctx, 1), 32, 0, ctx->stream>>>(sp->mesh->ctype, sp->order, L, tab);
  GT_LAUNCH(ctx, "k_tabulate");
  if (precision == GT_FP32)
    return elements_T<float>(sp, form, d_coef, nu, tab, L, (float*)Ke, nullptr, nullptr, nullptr, 1);
  return elements_T<double>(sp, form, d_coef, nu, tab, L, (double*)Ke, nullptr, nullptr, nullptr, 1);
}

// ---------------------------------------------------------------------------
// 4. scatter: G lanes own one block row; the row's column indices and
// accumulators live in shared memory; incidences are visited in ascending
// cell order with a group barrier between cells, so every entry is summed in
// the same order on every run.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int find_col(const int32_t* cols, int L, int32_t j) {
  int lo = 0, hi = L - 1;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (cols[mid] < j) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Load-vector entries of a block row: the element vectors of the row's
// incidences summed in one fixed order, shared by every kernel that sums
// them (k_scatter, k_scatter_kron, k_scatter_vec), so the load vector of
// assemble_vector is bitwise the one of assemble_matrix_and_vector: four
// partial sums s_j over the incidences ib + j, ib + j + 4, ... (ascending),
// combined as (s0 + s1) + (s2 + s3).
// s[cc] = s_j of components cc < BS of the element vectors (be: bs
// components per local node)
template <int BS>
__device__ __forceinline__ void load_partial(const int64_t ib, int64_t ie, int j, const int32_t* __restrict__ inc,
                                             int nn, int bs, const double* __restrict__ be, double* s) {
#pragma unroll
  for (int cc = 0; cc < BS; cc++) s[cc] = 0.0;
  for (int64_t k = ib + j; k < ie; k += 4) {
    int32_t cb = __ldg(inc + k);
    int32_t c = cb / nn, a = cb - c * nn;
#pragma unroll
    for (int cc = 0; cc < BS; cc++) s[cc] += __ldg(be + ((int64_t)c * nn + a) * bs + cc);
  }
}

// The same sum by lanes 0..3 of a row's group of G >= 4 lanes (lane j forms
// s_j; two butterfly steps combine them): one FP64 add per lane per four
// incidences, where a single lane summing in sequence would issue a warp
// FP64 instruction per incidence.  Every lane of the group gets the sums.
template <int BS>
__device__ __forceinline__ void row_load_sum(const int64_t ib, int64_t ie, const int32_t* __restrict__ inc, int nn,
                                             const double* __restrict__ be, int gl, unsigned gmask, double* out) {
  double s[BS];
  load_partial<BS>(ib, gl < 4 ? ie : ib, gl, inc, nn, BS, be, s);
#pragma unroll
  for (int cc = 0; cc < BS; cc++) {
    s[cc] += __shfl_xor_sync(gmask, s[cc], 1);
    s[cc] += __shfl_xor_sync(gmask, s[cc], 2);
    out[cc] = s[cc];
  }
}

// With be != nullptr the group also sums the element vectors of the row's
// incidences (row_load_sum), then lane 0 subtracts the Dirichlet lift of
// each incidence in ascending order (when xd), and writes bvec.
// (Scalar P1 tetrahedra, whose blocks are stored packed, take k_scatter_p1.)
template <int BS, int G, class TK, class TA>
__global__ void k_scatter(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                          const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                          const int32_t* __restrict__ cnd, int nn_arg, int64_t row_begin, int64_t row_end,
                          int lmax, const TK* __restrict__ Ke, double* __restrict__ v64, float* __restrict__ v32,
                          const double* __restrict__ be, double* __restrict__ bvec,
                          const double* __restrict__ xd) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  constexpr int RPW = 32 / G;  // rows per warp
  const int nn = nn_arg;
  const int nloc = nn * BS;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int sub = lane / G, gl = lane - sub * G;
  int slot = w * RPW + sub;
  TA* acc = (TA*)s_raw + (size_t)slot * lmax * BS * BS;
  int32_t* cols = (int32_t*)((TA*)s_raw + (size_t)(blockDim.x / G) * lmax * BS * BS) + (size_t)slot * lmax;
  int64_t r = row_begin + ((int64_t)blockIdx.x * (blockDim.x >> 5) + w) * RPW + sub;
  bool active = r < row_end;
  unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (sub * G));
  int64_t rb = 0;
  int L = 0;
  if (active) {
    rb = rowptr[r];
    L = (int)(rowptr[r + 1] - rb);
    for (int i = gl; i < L; i += G) cols[i] = colind[rb + i];
    for (int i = gl; i < L * BS * BS; i += G) acc[i] = (TA)0;
  }
  __syncwarp(gmask);
  if (active) {
    // lane gl owns local column node b = gl (nn <= G).  Incidences are taken
    // U at a time: the loads of all U are issued first (independent, in
    // flight together), then the U contributions are added in order with a
    // group barrier between cells, which keeps the summation order fixed.
    constexpr int U = BS == 1 ? 4 : 2;
    const int b = gl;
    const bool vec = be != nullptr && gl == 0;
    double bsum[BS];
    int64_t ib = inc_ptr[r], ie = inc_ptr[r + 1];
    if (be != nullptr) {
      row_load_sum<BS>(ib, ie, inc, nn, be, gl, gmask, bsum);
    } else {
#pragma unroll
      for (int cc = 0; cc < BS; cc++) bsum[cc] = 0.0;
    }
    for (int64_t k0 = ib; k0 < ie; k0 += U) {
      int32_t jj[U];
      TA kv[U][BS * BS];
#pragma unroll
      for (int u = 0; u < U; u++) {
        jj[u] = 0;
        int64_t k = k0 + u;
        if (k < ie && b < nn) {
          int32_t cb = __ldg(inc + k);
          int32_t c = cb / nn, a = cb - c * nn;
          jj[u] = __ldg(cnd + (int64_t)c * nn + b);
          const TK* Krow = Ke + (int64_t)c * nloc * nloc + (int64_t)(a * BS) * nloc + b * BS;
#pragma unroll
          for (int cc = 0; cc < BS; cc++)
#pragma unroll
            for (int dd = 0; dd < BS; dd++) kv[u][cc * BS + dd] = (TA)__ldg(Krow + cc * nloc + dd);
        }
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (jj[u] > 0) {
          int p = find_col(cols, L, jj[u] - 1);
#pragma unroll
          for (int e = 0; e < BS * BS; e++) acc[p * BS * BS + e] += kv[u][e];
        }
        if (xd != nullptr && be != nullptr) {
          // Dirichlet lift b -= Ad xd: this incidence's Dirichlet columns,
          // summed over the group's lanes in a fixed butterfly
          double lv[BS];
#pragma unroll
          for (int cc = 0; cc < BS; cc++) lv[cc] = 0.0;
          if (jj[u] < 0)
#pragma unroll
            for (int cc = 0; cc < BS; cc++)
#pragma unroll
              for (int dd = 0; dd < BS; dd++)
                lv[cc] += (double)kv[u][cc * BS + dd] * __ldg(xd + (int64_t)(-jj[u] - 1) * BS + dd);
#pragma unroll
          for (int cc = 0; cc < BS; cc++) {
#pragma unroll
            for (int o = G >> 1; o; o >>= 1) lv[cc] += __shfl_xor_sync(gmask, lv[cc], o);
            if (gl == 0) bsum[cc] -= lv[cc];
          }
        }
        __syncwarp(gmask);
      }
    }
    int64_t ob = rb * BS * BS;
    for (int i = gl; i < L * BS * BS; i += G) {
      TA v = acc[i];
      if (v64) v64[ob + i] = (double)v;
      if (v32) v32[ob + i] = (float)v;
    }
    if (vec)
#pragma unroll
      for (int cc = 0; cc < BS; cc++) bvec[r * BS + cc] = bsum[cc];
  }
}

// Element-block entries and row accumulators of the P1 scatter: FP64 or
// FP32 numbers, or double-float pairs (the double-float element kernel's
// entries, summed as pairs on the FP32 pipes and rounded to FP64 once per
// CSR value).
template <class T>
__device__ __forceinline__ T ke_load(const T* p) { return __ldg(p); }
template <>
__device__ __forceinline__ dfl ke_load<dfl>(const dfl* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return {v.x, v.y};
}
__device__ __forceinline__ void acc_add(double& a, double v) { a += v; }
__device__ __forceinline__ void acc_add(float& a, float v) { a += v; }
__device__ __forceinline__ void acc_add(dfl& a, dfl v) { a = df_add_sloppy(a, v); }
__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ double to_f64(float v) { return (double)v; }
__device__ __forceinline__ double to_f64(dfl v) { return df_to_double(v); }
__device__ __forceinline__ float to_f32(double v) { return (float)v; }
__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(dfl v) { return (float)df_to_double(v); }

// Scalar P1 tetrahedra (packed blocks: the upper triangle of the symmetric
// 4 x 4 block, 10 entries per cell): the row-owner scatter of k_scatter,
// specialised.  Four lanes own a row, lane b the local column node b of
// every incidence.  Incidences are taken U at a time: their loads are
// issued together; their column positions come from branchless binary
// searches advanced in lock step (the row's length fixes the number of
// steps, so the U searches overlap instead of running one after the other);
// then the U contributions are added in ascending incidence order with a
// group barrier between them -- the summation order of k_scatter, so the
// values are bitwise those of the generic kernel.  LIFT (the Dirichlet lift
// b -= Ad xd) is a compile-time choice, so the common case carries none of
// its FP64 code.  NB > 0: every row has at most 2^NB columns, the slot
// holds 2^NB of them (the tail padded with INT_MAX) and the search takes NB
// steps of fixed width 2^(NB-1), ..., 1 -- unrolled, constant offsets --
// instead of the row-length loop (NB = 0); same positions, same values.
// The slot strides set the shared-memory bank conflicts: the eight rows of a
// warp are consecutive DOFs, whose incidences on a structured mesh hit the
// same column positions at the same step, so the row slots must not map
// those positions onto one bank.  Column slots 2^NB + 5 words apart and
// accumulator slots 2^NB + 4 entries apart (8-byte entries: the four rows of
// a half warp start 0, 4, 8, 12 bank pairs apart) take, on the P1 Kuhn-cube
// pattern, 1.53 wavefronts per search load and 3.9 per accumulator access,
// against 2.5 and 5.2 with both 2^NB + 1 apart and 4.0 and 7.5 with 2^NB.  Its first two steps compare with three columns
// held in registers (the only ones they can read), so each search reads
// shared memory NB - 2 times: the kernel is bound by the L1 data pipe
// (shared-memory wavefronts of the searches and accumulators plus the
// gathers' wavefronts), not by DRAM.
template <class TK, class TA, bool LIFT, int NB>
__global__ void __launch_bounds__(128) k_scatter_p1(const int64_t* __restrict__ rowptr,
                                                    const int32_t* __restrict__ colind,
                                                    const int64_t* __restrict__ inc_ptr,
                                                    const int32_t* __restrict__ inc, const int32_t* __restrict__ cnd,
                                                    int /* nodes per cell: 4 */, int64_t row_begin, int64_t row_end,
                                                    int lmax,
                                                    const TK* __restrict__ Ke, double* __restrict__ v64,
                                                    float* __restrict__ v32, const double* __restrict__ be,
                                                    double* __restrict__ bvec, const double* __restrict__ xd) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  constexpr int G = 4, RPW = 8, U = 8;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int sub = lane >> 2, b = lane & 3;
  const int slot = w * RPW + sub;
  // accumulator slots lmax entries apart, column slots one more (NB > 0)
  const int cstride = NB > 0 ? lmax + 1 : lmax;
  TA* acc = (TA*)s_raw + (size_t)slot * lmax;
  int32_t* cols = (int32_t*)((TA*)s_raw + (size_t)(blockDim.x / G) * lmax) + (size_t)slot * cstride;
  const int64_t r = row_begin + ((int64_t)blockIdx.x * (blockDim.x >> 5) + w) * RPW + sub;
  if (r >= row_end) return;  // the group's four lanes leave together
  const unsigned gmask = 0xfu << (sub * G);
  // packed offset of entry (a, b) for this lane's b, one nibble per a:
  // (min, max) of the pair in the row-by-row upper triangle
  unsigned offs = 0;
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const int lo = a < b ? a : b, hi = a ^ b ^ lo;
    offs |= (unsigned)(lo * 4 - ((lo * (lo - 1)) >> 1) + (hi - lo)) << (4 * a);
  }
  const int64_t rb = rowptr[r];
  const int L = (int)(rowptr[r + 1] - rb);
  for (int i = b; i < L; i += G) {
    cols[i] = colind[rb + i];
    acc[i] = TA{};
  }
  if constexpr (NB > 0)
    for (int i = L + b; i < (1 << NB); i += G) cols[i] = INT_MAX;  // above every key
  __syncwarp(gmask);
  // the columns of the first two search steps: H1, then H1 - H2 or H1 + H2
  constexpr int H1 = NB > 0 ? 1 << (NB - 1) : 1, H2 = NB > 1 ? 1 << (NB - 2) : 1;
  int32_t c_mid = 0, c_lo = 0, c_hi = 0;
  if constexpr (NB > 1) {
    c_mid = cols[H1];
    c_lo = cols[H1 - H2];
    c_hi = cols[H1 + H2];
  }
  const int64_t ib = inc_ptr[r], ie = inc_ptr[r + 1];
  double bsum = 0.0;
  if (be != nullptr) row_load_sum<1>(ib, ie, inc, 4, be, b, gmask, &bsum);
  for (int64_t k0 = ib; k0 < ie; k0 += U) {
    int32_t jj[U], key[U];
    int pos[U];
    TA kv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      jj[u] = 0;
      kv[u] = TA{};
      if (k0 + u < ie) {
        const int32_t cb = __ldg(inc + k0 + u);
        const int32_t c = cb >> 2, a = cb & 3;
        jj[u] = __ldg(cnd + (int64_t)c * 4 + b);
        kv[u] = (TA)ke_load(Ke + (int64_t)c * 10 + ((offs >> (4 * a)) & 15u));
      }
      key[u] = jj[u] > 0 ? jj[u] - 1 : INT_MIN;  // INT_MIN: stays at position 0, unused
      pos[u] = 0;
    }
    // last position whose column is <= key: the column's own position
    if constexpr (NB > 1) {
#pragma unroll
      for (int u = 0; u < U; u++) {
        const bool up = c_mid <= key[u];
        pos[u] = up ? H1 : 0;
        if ((up ? c_hi : c_lo) <= key[u]) pos[u] += H2;
      }
#pragma unroll
      for (int half = H2 >> 1; half > 0; half >>= 1)
#pragma unroll
        for (int u = 0; u < U; u++) pos[u] = cols[pos[u] + half] <= key[u] ? pos[u] + half : pos[u];
    } else if constexpr (NB > 0) {
#pragma unroll
      for (int half = 1 << (NB - 1); half > 0; half >>= 1)
#pragma unroll
        for (int u = 0; u < U; u++) pos[u] = cols[pos[u] + half] <= key[u] ? pos[u] + half : pos[u];
    } else {
      for (int n = L; n > 1;) {
        const int half = n >> 1;
#pragma unroll
        for (int u = 0; u < U; u++) pos[u] = cols[pos[u] + half] <= key[u] ? pos[u] + half : pos[u];
        n -= half;
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (jj[u] > 0) acc_add(acc[pos[u]], kv[u]);
      if constexpr (LIFT) {
        double lv = 0.0;
        if (jj[u] < 0) lv += to_f64(kv[u]) * __ldg(xd - jj[u] - 1);
        lv += __shfl_xor_sync(gmask, lv, 2);
        lv += __shfl_xor_sync(gmask, lv, 1);
        if (b == 0) bsum -= lv;
      }
      __syncwarp(gmask);
    }
  }
  for (int i = b; i < L; i += G) {
    const TA v = acc[i];
    if (v64) v64[rb + i] = to_f64(v);
    if (v32) v32[rb + i] = to_f32(v);
  }
  if (be != nullptr && b == 0) bvec[r] = bsum;
}

template <int BS, class TK, class TA>
static int launch_scatter(Matrix* A, const TK* Ke, double* v64, float* v32, const double* be, double* bvec,
                          const double* xd, int64_t r0, int64_t r1) {
  const Space* sp = A->space;
  Ctx* ctx = ctx_of(sp);
  int nn = sp->nn;
  // row slots an odd number of entries apart: the groups of a warp, all at
  // the same step of their rows, then read different banks
  int lmax = (A->max_row > 0 ? A->max_row : 1) | 1;
  // the P1 kernel's fixed-step search: slots of 16 or 32 columns, the
  // accumulator slots 2^NB + 4 entries apart (the column slots one more)
  const int p1_nb = (BS == 1 && ke_packed(sp)) ? (A->max_row <= 16 ? 4 : (A->max_row <= 32 ? 5 : 0)) : 0;
  if (p1_nb > 0) lmax = (1 << p1_nb) + 4;
  auto go = [&](auto Gtag) -> int {
    constexpr int G = decltype(Gtag)::value;
    constexpr int RPW = 32 / G;
    int warps = 4;
    size_t per_row = (size_t)lmax * (BS * BS * sizeof(TA) + sizeof(int32_t)) + (p1_nb > 0 ? sizeof(int32_t) : 0);
    while (warps > 1 && (size_t)warps * RPW * per_row > 96 * 1024) warps >>= 1;
    size_t smem = (size_t)warps * RPW * per_row;
    if (smem > 200 * 1024) return set_error(ctx, GT_ERR_UNSUPPORTED, "sparsity row too wide for the scatter kernel");
    int64_t rows_per_block = (int64_t)warps * RPW;
    int64_t grid = (r1 - r0 + rows_per_block - 1) / rows_per_block;
    auto launch = [&](auto kern) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      kern<<<GT_KC(ctx, (unsigned)(grid > 0 ? grid : 1)), warps * 32, smem, ctx->stream>>>(
          A->rowptr, A->colind, A->inc_ptr, A->inc, sp->cell_ndofs, nn, r0, r1, lmax, Ke, v64, v32, be, bvec, xd);
    };
    bool done = false;
    if constexpr (BS == 1 && G == 4) {
      if (ke_packed(sp)) {
        const bool lift = xd != nullptr && be != nullptr;
        if (p1_nb == 4)
          lift ? launch(k_scatter_p1<TK, TA, true, 4>) : launch(k_scatter_p1<TK, TA, false, 4>);
        else if (p1_nb == 5)
          lift ? launch(k_scatter_p1<TK, TA, true, 5>) : launch(k_scatter_p1<TK, TA, false, 5>);
        else
          lift ? launch(k_scatter_p1<TK, TA, true, 0>) : launch(k_scatter_p1<TK, TA, false, 0>);
        done = true;
      }
    }
    if constexpr (!std::is_same<TK, dfl>::value) {
      if (!done) launch(k_scatter<BS, G, TK, TA>);
    }
    GT_LAUNCH(ctx, "k_scatter");
    return GT_OK;
  };
  if (nn <= 4) return go(std::integral_constant<int, 4>());
  if (nn <= 8) return go(std::integral_constant<int, 8>());
  if (nn <= 16) return go(std::integral_constant<int, 16>());
  return go(std::integral_constant<int, 32>());
}

int scatter_matrix(Matrix* A, const void* Ke, int ke_precision, int out_precision, const double* be, double* bvec,
                   const double* xd, int64_t r0, int64_t r1) {
  if (r1 < 0) r1 = A->nbrows;
  matrix_values_changed(A);
  double* v64 = (out_precision == GT_FP64 || out_precision == GT_MIXED) ? A->val64 : nullptr;
  float* v32 = (out_precision == GT_FP32 || out_precision == GT_MIXED) ? A->val32 : nullptr;
  int bs = A->bs;
  if (ke_precision == GT_FP32) {
    const float* K = (const float*)Ke;
    if (bs == 1) return launch_scatter<1, float, float>(A, K, v64, v32, be, bvec, xd, r0, r1);
    if (bs == 2) return launch_scatter<2, float, float>(A, K, v64, v32, be, bvec, xd, r0, r1);
    return launch_scatter<3, float, float>(A, K, v64, v32, be, bvec, xd, r0, r1);
  }
  // FP64-valued packed P1 blocks from the double-float element kernel are
  // double-float pairs
  if (bs == 1 && ke_packed(A->space) && ctx_of(A->space)->p1_dfloat)
    return launch_scatter<1, dfl, dfl>(A, (const dfl*)Ke, v64, v32, be, bvec, xd, r0, r1);
  const double* K = (const double*)Ke;
  if (bs == 1) return launch_scatter<1, double, double>(A, K, v64, v32, be, bvec, xd, r0, r1);
  if (bs == 2) return launch_scatter<2, double, double>(A, K, v64, v32, be, bvec, xd, r0, r1);
  return launch_scatter<3, double, double>(A, K, v64, v32, be, bvec, xd, r0, r1);
}

// ---------------------------------------------------------------------------
// Sum-factorised path for affine quadrilaterals / hexahedra (Q1, Q2).
// On an affine cell J is constant, so with tensor-product shape functions
// and tensor Gauss quadrature the reference's quadrature sum factorises:
//   sum_q w_q dV gradref_n[k] gradref_m[l] = |det J| prod_e F_e(n_e, m_e)
// with F_e one of the 1-D matrices M = sum w L_i L_j, Dm = sum w L'_i L_j,
// Kd = sum w L'_i L'_j (Kd on e = k = l, Dm on e = k, Dm^T on e = l, else M).
// The physical gradients are J^-T gradref, so an element-matrix block is a
// few products of 1-D entries and the per-cell J^-1 -- cheap enough to
// compute inside the row-owner scatter for every (row, cell, column node),
// so no element matrix ever goes through HBM.
//   k_geom_affine: FP64 J, det, J^-1 per cell (+ the load vector), affinity
//                  check; stores G[c] = {J^-1 or the metric J^-1 J^-T, scale}
//   k_scatter_kron: like k_scatter, with blocks computed from G and the
//                  1-D tables instead of read from Ke
// ---------------------------------------------------------------------------
constexpr int GSTRIDE = 10;  // per-cell geometry record: 9 + 1 values

__device__ void lagrange_table_1d(int order, double* M, double* Dm, double* Kd, double* m1) {
  int n1 = order + 1;
  double g[3], gw[3];
  if (n1 == 2) {
    double s = 0.5 / sqrt(3.0);
    g[0] = 0.5 - s; g[1] = 0.5 + s; gw[0] = gw[1] = 0.5;
  } else {
    double s = 0.5 * sqrt(0.6);
    g[0] = 0.5 - s; g[1] = 0.5; g[2] = 0.5 + s;
    gw[0] = 5.0 / 18.0; gw[1] = 8.0 / 18.0; gw[2] = 5.0 / 18.0;
  }
  for (int i = 0; i < 9; i++) M[i] = Dm[i] = Kd[i] = 0.0;
  for (int i = 0; i < 3; i++) m1[i] = 0.0;
  for (int q = 0; q < n1; q++) {
    double v[3], dv[3];
    lagrange1d(order, g[q], v, dv);
    for (int i = 0; i < n1; i++) {
      m1[i] += gw[q] * v[i];
      for (int j = 0; j < n1; j++) {
        M[i * 3 + j] += gw[q] * v[i] * v[j];
        Dm[i * 3 + j] += gw[q] * dv[i] * v[j];
        Kd[i * 3 + j] += gw[q] * dv[i] * dv[j];
      }
    }
  }
}

// geometry record of one affine QUAD4/HEX8 cell: J^-1 (elasticity) or the
// metric J^-1 J^-T (Laplacian) in gv[0..D*D), |det J| and det J; false when
// some node is off the affine map x0 + sum_d bit_d(n) J[:, d]
template <int D, int NV>
__device__ __forceinline__ bool affine_record(const double* __restrict__ coords, const int32_t* __restrict__ cell_nodes,
                                              int64_t c, int form, double (&gv)[GSTRIDE], double& adet,
                                              double& det) {
  double x[NV][D];
#pragma unroll
  for (int n = 0; n < NV; n++) {
    const double* p = coords + (int64_t)cell_nodes[c * NV + n] * D;
#pragma unroll
    for (int d = 0; d < D; d++) x[n][d] = p[d];
  }
  double J[D][D];
#pragma unroll
  for (int i = 0; i < D; i++)
#pragma unroll
    for (int d = 0; d < D; d++) J[i][d] = x[1 << d][i] - x[0][i];
  double hmax = 0.0;
#pragma unroll
  for (int i = 0; i < D; i++)
#pragma unroll
    for (int d = 0; d < D; d++) hmax = fmax(hmax, fabs(J[i][d]));
  bool affine = true;
#pragma unroll
  for (int n = 3; n < NV; n++) {
#pragma unroll
    for (int i = 0; i < D; i++) {
      double pred = x[0][i];
#pragma unroll
      for (int d = 0; d < D; d++)
        if ((n >> d) & 1) pred += J[i][d];
      if (fabs(x[n][i] - pred) > 1e-13 * hmax) affine = false;
    }
  }
  double inv[D][D];
  if (D == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    double r = recip_nr2(det);
    inv[0][0] = J[1][1] * r; inv[0][1] = -J[0][1] * r;
    inv[1][0] = -J[1][0] * r; inv[1][1] = J[0][0] * r;
  } else {
    double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    double r = recip_nr2(det);
    inv[0][0] = c00 * r; inv[1][0] = c01 * r; inv[2][0] = c02 * r;
    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
  }
  adet = fabs(det);
#pragma unroll
  for (int i = 0; i < GSTRIDE; i++) gv[i] = 0.0;
  if (form == GT_LAPLACE) {
    // metric Gm[k][l] = sum_c J^-1[k][c] J^-1[l][c]
#pragma unroll
    for (int k = 0; k < D; k++)
#pragma unroll
      for (int l = 0; l < D; l++) {
        double s = 0.0;
#pragma unroll
        for (int cc = 0; cc < D; cc++) s += inv[k][cc] * inv[l][cc];
        gv[k * D + l] = s;
      }
  } else {
#pragma unroll
    for (int k = 0; k < D; k++)
#pragma unroll
      for (int l = 0; l < D; l++) gv[k * D + l] = inv[k][l];
  }
  return affine;
}

// the record of cell 0: the reference of the uniformity test
// (gref[0..GSTRIDE-1) the record, gref[GSTRIDE-1] |det J|)
template <int D, int NV>
__global__ void k_geom_ref(const double* __restrict__ coords, const int32_t* __restrict__ cell_nodes, int form,
                           double* __restrict__ gref) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double gv[GSTRIDE], adet, det;
  affine_record<D, NV>(coords, cell_nodes, 0, form, gv, adet, det);
  gv[GSTRIDE - 1] = adet;
#pragma unroll
  for (int i = 0; i < GSTRIDE; i++) gref[i] = gv[i];
}

// per-cell records G[c] = {record, scale = |det J| coef_c} (+ the load
// vector), affinity check, and -- with gref -- the uniformity test: a cell
// whose record and |det J| differ from cell 0's by more than 1e-13 of the
// largest record entry (of |det J|) sets *nonuniform
template <int D, int NV>
__global__ void __launch_bounds__(256) k_geom_affine(const double* __restrict__ coords,
                                                     const int32_t* __restrict__ cell_nodes,
                                                     const double* __restrict__ coef, int form, int order,
                                                     int64_t ncells, int nn, int bs, void* __restrict__ Gout, int g64,
                                                     double* __restrict__ be, const double* __restrict__ fsrc,
                                                     const double* __restrict__ scoef, uint32_t* nonaffine,
                                                     uint32_t* err, const double* __restrict__ gref,
                                                     uint32_t* nonuniform) {
  __shared__ double s_m1[3];
  if (threadIdx.x == 0) {
    double M[9], Dm[9], Kd[9];
    lagrange_table_1d(order, M, Dm, Kd, s_m1);
  }
  __syncthreads();
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  double gv[GSTRIDE], adet, det;
  if (!affine_record<D, NV>(coords, cell_nodes, c, form, gv, adet, det)) atomicOr(nonaffine, 1u);
  if (!(det != 0.0)) atomicOr(err, DEV_ERR_DEGENERATE);
  if (gref) {
    double gm = 0.0;
#pragma unroll
    for (int i = 0; i < D * D; i++) gm = fmax(gm, fabs(gref[i]));
    bool same = fabs(adet - gref[GSTRIDE - 1]) <= 1e-13 * gref[GSTRIDE - 1];
#pragma unroll
    for (int i = 0; i < D * D; i++) same = same && fabs(gv[i] - gref[i]) <= 1e-13 * gm;
    if (!same) atomicOr(nonuniform, 1u);
  }
  const double scale = adet * (coef ? coef[c] : 1.0);
  gv[GSTRIDE - 1] = scale;
  if (g64) {
    double* G = (double*)Gout + c * GSTRIDE;
#pragma unroll
    for (int i = 0; i < GSTRIDE; i++) G[i] = gv[i];
  } else {
    float* G = (float*)Gout + c * GSTRIDE;
#pragma unroll
    for (int i = 0; i < GSTRIDE; i++) G[i] = (float)gv[i];
  }
  if (be) {
    int m1 = order + 1;
    double sc = (scoef ? scoef[c] : 1.0) * adet;
    for (int n = 0; n < nn; n++) {
      int e0 = n % m1, e1 = (n / m1) % m1, e2 = n / (m1 * m1);
      double w = s_m1[e0] * s_m1[e1] * (D == 3 ? s_m1[e2] : 1.0);
      for (int k = 0; k < bs; k++) be[(c * nn + n) * bs + k] = sc * fsrc[k] * w;
    }
  }
}

// one BSxBS block (row node with 1-D indices na, column node nb) of an
// affine cell from its geometry record g and the 1-D tables
template <int D, int BS, int FORM, class T>
__device__ __forceinline__ void kron_block(const int* na, const int* nb, const T* g, const T* M, const T* Dm,
                                           const T* Kd, T lamf, T muf, T (&blk)[BS][BS]) {
  const T scale = g[GSTRIDE - 1];
  if constexpr (FORM == GT_MASS) {
    T v = scale;
#pragma unroll
    for (int e = 0; e < D; e++) v *= M[na[e] * 3 + nb[e]];
#pragma unroll
    for (int a = 0; a < BS; a++)
#pragma unroll
      for (int b = 0; b < BS; b++) blk[a][b] = a == b ? v : (T)0;
  } else {
  // reference integrals I[k][l] = prod_e F_e
  T I[D][D];
#pragma unroll
  for (int k = 0; k < D; k++)
#pragma unroll
    for (int l = 0; l < D; l++) {
      T v = (T)1;
#pragma unroll
      for (int e = 0; e < D; e++) {
        int i = na[e], j = nb[e];
        T f = (e == k && e == l) ? Kd[i * 3 + j] : (e == k) ? Dm[i * 3 + j] : (e == l) ? Dm[j * 3 + i] : M[i * 3 + j];
        v *= f;
      }
      I[k][l] = v;
    }
  if constexpr (FORM == GT_LAPLACE) {
    T s = (T)0;
#pragma unroll
    for (int k = 0; k < D; k++)
#pragma unroll
      for (int l = 0; l < D; l++) s += g[k * D + l] * I[k][l];
    s *= scale;
#pragma unroll
    for (int a = 0; a < BS; a++)
#pragma unroll
      for (int b = 0; b < BS; b++) blk[a][b] = a == b ? s : (T)0;
  } else {
  // elasticity: A[c][d] = scale sum_kl J^-1[k][c] J^-1[l][d] I[k][l]
  T t1[D][D], A[D][D];
#pragma unroll
  for (int k = 0; k < D; k++)
#pragma unroll
    for (int d = 0; d < D; d++) {
      T s = (T)0;
#pragma unroll
      for (int l = 0; l < D; l++) s += I[k][l] * g[l * D + d];
      t1[k][d] = s;
    }
  T tr = (T)0;
#pragma unroll
  for (int c = 0; c < D; c++)
#pragma unroll
    for (int d = 0; d < D; d++) {
      T s = (T)0;
#pragma unroll
      for (int k = 0; k < D; k++) s += g[k * D + c] * t1[k][d];
      A[c][d] = s * scale;
    }
#pragma unroll
  for (int c = 0; c < D; c++) tr += A[c][c];
#pragma unroll
  for (int a = 0; a < BS; a++)
#pragma unroll
    for (int b = 0; b < BS; b++) blk[a][b] = lamf * A[a][b] + muf * A[b][a] + (a == b ? muf * tr : (T)0);
  }  // elasticity
  }  // not mass
}

template <int D, int ORDER, int BS, int FORM, int G, class T, class TA>
__global__ void k_scatter_kron(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                               const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                               const int32_t* __restrict__ cnd, int64_t nrows, int lmax, const T* __restrict__ Gc,
                               T lamf, T muf, double* __restrict__ v64, float* __restrict__ v32,
                               const double* __restrict__ be, double* __restrict__ bvec, const double* __restrict__ xd) {
  constexpr int M1 = ORDER + 1;
  constexpr int NN = D == 2 ? M1 * M1 : M1 * M1 * M1;
  constexpr int RPW = 32 / G;
  extern __shared__ __align__(16) unsigned char s_raw[];
  __shared__ T s_M[9], s_D[9], s_K[9];
  if (threadIdx.x == 0) {
    double M[9], Dm[9], Kd[9], m1[3];
    lagrange_table_1d(ORDER, M, Dm, Kd, m1);
    for (int i = 0; i < 9; i++) { s_M[i] = (T)M[i]; s_D[i] = (T)Dm[i]; s_K[i] = (T)Kd[i]; }
  }
  __syncthreads();
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int sub = lane / G, gl = lane - sub * G;
  int slot = w * RPW + sub;
  TA* acc = (TA*)s_raw + (size_t)slot * lmax * BS * BS;
  int32_t* cols = (int32_t*)((TA*)s_raw + (size_t)(blockDim.x / G) * lmax * BS * BS) + (size_t)slot * lmax;
  int64_t r = ((int64_t)blockIdx.x * (blockDim.x >> 5) + w) * RPW + sub;
  bool active = r < nrows;
  unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (sub * G));
  int64_t rb = 0;
  int L = 0;
  if (active) {
    rb = rowptr[r];
    L = (int)(rowptr[r + 1] - rb);
    for (int i = gl; i < L; i += G) cols[i] = colind[rb + i];
    for (int i = gl; i < L * BS * BS; i += G) acc[i] = (TA)0;
  }
  __syncwarp(gmask);
  if (active) {
    const int b = gl;
    int nbi[3] = {b % M1, (b / M1) % M1, b / (M1 * M1)};
    // with be: the group also sums the load vector of the row (row_load_sum),
    // and lane 0 subtracts the Dirichlet lift when xd
    const bool vec = be != nullptr && gl == 0;
    const bool lift = be != nullptr && xd != nullptr;
    double bsum[BS];
    int64_t ib = inc_ptr[r], ie = inc_ptr[r + 1];
    if (be != nullptr) {
      row_load_sum<BS>(ib, ie, inc, NN, be, gl, gmask, bsum);
    } else {
#pragma unroll
      for (int cc = 0; cc < BS; cc++) bsum[cc] = 0.0;
    }
    for (int64_t k = ib; k < ie; k++) {
      int32_t cb = __ldg(inc + k);
      int32_t c = cb / NN, a = cb - c * NN;
      double lv[BS];
#pragma unroll
      for (int cc = 0; cc < BS; cc++) lv[cc] = 0.0;
      if (b < NN) {
        int32_t j = __ldg(cnd + (int64_t)c * NN + b);
        if (j > 0 || (j < 0 && lift)) {
          T g[GSTRIDE];
#pragma unroll
          for (int i = 0; i < GSTRIDE; i++) g[i] = __ldg(Gc + (int64_t)c * GSTRIDE + i);
          int nai[3] = {a % M1, (a / M1) % M1, a / (M1 * M1)};
          T blk[BS][BS];
          kron_block<D, BS, FORM, T>(nai, nbi, g, s_M, s_D, s_K, lamf, muf, blk);
          if (j > 0) {
            int p = find_col(cols, L, j - 1);
#pragma unroll
            for (int cc = 0; cc < BS; cc++)
#pragma unroll
              for (int dd = 0; dd < BS; dd++) acc[(p * BS + cc) * BS + dd] += (TA)blk[cc][dd];
          } else {
#pragma unroll
            for (int cc = 0; cc < BS; cc++)
#pragma unroll
              for (int dd = 0; dd < BS; dd++) lv[cc] += (double)blk[cc][dd] * __ldg(xd + (int64_t)(-j - 1) * BS + dd);
          }
        }
      }
      if (lift)
#pragma unroll
        for (int cc = 0; cc < BS; cc++) {
#pragma unroll
          for (int o = G >> 1; o; o >>= 1) lv[cc] += __shfl_xor_sync(gmask, lv[cc], o);
          if (gl == 0) bsum[cc] -= lv[cc];
        }
      __syncwarp(gmask);
    }
    int64_t ob = rb * BS * BS;
    for (int i = gl; i < L * BS * BS; i += G) {
      TA v = acc[i];
      if (v64) v64[ob + i] = (double)v;
      if (v32) v32[ob + i] = (float)v;
    }
    if (vec)
#pragma unroll
      for (int cc = 0; cc < BS; cc++) bvec[r * BS + cc] = bsum[cc];
  }
}

// Uniform geometry: every cell has the reference record (cell 0's), so an
// element block is scale_c x Kref[a][b] with Kref the unit-scale block of
// the reference record and scale_c = |det J| coef_c.  k_kref computes Kref
// once (kron_block: FP64 for FP64 values, FP32 for FP32 values) into global
// memory; k_scatter_uniform is persistent: each CTA copies Kref into shared
// memory once and then loops over row groups, so the per-(row, cell, column
// node) work is BS*BS multiply-adds instead of a kron_block.  Otherwise as
// k_scatter_kron (row owner, incidences in ascending cell order, load vector
// and Dirichlet lift in the same pass).
template <int D, int ORDER, int BS, int FORM, class T>
__global__ void k_kref(const double* __restrict__ gref, T lamf, T muf, T* __restrict__ kref) {
  constexpr int M1 = ORDER + 1;
  constexpr int NN = D == 2 ? M1 * M1 : M1 * M1 * M1;
  __shared__ T s_M[9], s_D[9], s_K[9];
  if (threadIdx.x == 0) {
    double M[9], Dm[9], Kd[9], m1[3];
    lagrange_table_1d(ORDER, M, Dm, Kd, m1);
    for (int i = 0; i < 9; i++) { s_M[i] = (T)M[i]; s_D[i] = (T)Dm[i]; s_K[i] = (T)Kd[i]; }
  }
  __syncthreads();
  const int ab = blockIdx.x * blockDim.x + threadIdx.x;
  if (ab >= NN * NN) return;
  T g[GSTRIDE];
#pragma unroll
  for (int i = 0; i < GSTRIDE - 1; i++) g[i] = (T)gref[i];
  g[GSTRIDE - 1] = (T)1;
  const int a = ab / NN, b = ab - (ab / NN) * NN;
  int na[3] = {a % M1, (a / M1) % M1, a / (M1 * M1)};
  int nb[3] = {b % M1, (b / M1) % M1, b / (M1 * M1)};
  T blk[BS][BS];
  kron_block<D, BS, FORM, T>(na, nb, g, s_M, s_D, s_K, lamf, muf, blk);
#pragma unroll
  for (int cc = 0; cc < BS; cc++)
#pragma unroll
    for (int dd = 0; dd < BS; dd++) kref[(size_t)ab * BS * BS + cc * BS + dd] = blk[cc][dd];
}

template <int D, int ORDER, int BS, int G, class T, bool LIFT>
__global__ void k_scatter_uniform(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                  const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                  const int32_t* __restrict__ cnd, int64_t nrows, int lmax,
                                  const T* __restrict__ kref, const double* __restrict__ gref,
                                  const double* __restrict__ coef, double* __restrict__ v64, float* __restrict__ v32,
                                  const double* __restrict__ be, double* __restrict__ bvec,
                                  const double* __restrict__ xd) {
  constexpr int M1 = ORDER + 1;
  constexpr int NN = D == 2 ? M1 * M1 : M1 * M1 * M1;
  constexpr int RPW = 32 / G;
  constexpr int KB = BS * BS;
  constexpr int KREF_N = NN * NN * KB;
  constexpr size_t KREF_BYTES = ((size_t)KREF_N * sizeof(T) + 15) & ~size_t(15);
  constexpr int PF = G < 8 ? G : 8;  // incidences fetched ahead per row
  extern __shared__ __align__(16) unsigned char s_raw[];
  T* s_ref = (T*)s_raw;
  for (int i = threadIdx.x; i < KREF_N; i += blockDim.x) s_ref[i] = __ldg(kref + i);
  __syncthreads();
  const double adet = __ldg(gref + GSTRIDE - 1);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int sub = lane / G, gl = lane - sub * G;
  const int slot = w * RPW + sub;
  T* acc = (T*)(s_raw + KREF_BYTES) + (size_t)slot * lmax * KB;
  int32_t* cols = (int32_t*)((T*)(s_raw + KREF_BYTES) + (size_t)(blockDim.x / G) * lmax * KB) + (size_t)slot * lmax;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (sub * G));
  const bool vec = be != nullptr && gl == 0;
  const int b = gl;
  const int64_t nblk = (nrows + (int64_t)nw * RPW - 1) / ((int64_t)nw * RPW);
  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t r = (blk * nw + w) * RPW + sub;
    if (r >= nrows) continue;  // the group's lanes all skip together
    const int64_t rb = rowptr[r];
    const int L = (int)(rowptr[r + 1] - rb);
    for (int i = gl; i < L; i += G) cols[i] = colind[rb + i];
    for (int i = gl; i < L * KB; i += G) acc[i] = (T)0;
    __syncwarp(gmask);
    double bsum[BS];
    const int64_t ib = inc_ptr[r], ie = inc_ptr[r + 1];
    if (be != nullptr) {
      row_load_sum<BS>(ib, ie, inc, NN, be, gl, gmask, bsum);
    } else {
#pragma unroll
      for (int cc = 0; cc < BS; cc++) bsum[cc] = 0.0;
    }
    // the row's first PF incidences (at most 2^D on a structured mesh) are
    // fetched up front: their cells, each lane's column DOF and the cells'
    // scales are loads in flight together, and the column positions are
    // independent searches, so the summation loop below waits on no global
    // load; later incidences (a node in more than PF cells) load in the loop
    const int nin = (int)(ie - ib);
    const int32_t my_cb = gl < nin ? __ldg(inc + ib + gl) : 0;
    // each incidence's scale |det J| coef_c computed by one lane and handed
    // to the group by shuffles (a conversion per lane would load the FP64
    // pipe, which also converts FP64 to FP32)
    const T my_sc = (T)(adet * ((coef && gl < nin) ? __ldg(coef + my_cb / NN) : 1.0));
    int32_t cbk[PF], jk[PF], pk[PF];
    T sck[PF];
#pragma unroll
    for (int k = 0; k < PF; k++) {
      cbk[k] = __shfl_sync(gmask, my_cb, k, G);
      const int32_t c = cbk[k] / NN;
      jk[k] = (k < nin && b < NN) ? __ldg(cnd + (int64_t)c * NN + b) : 0;
      sck[k] = __shfl_sync(gmask, my_sc, k, G);
    }
#pragma unroll
    for (int k = 0; k < PF; k++) pk[k] = jk[k] > 0 ? find_col(cols, L, jk[k] - 1) : -1;
    // incidence cb's block: row node a, this lane's column node b (column
    // DOF j, position p), scale sc; then the group barrier that keeps the
    // summation order
    auto contribute = [&](int32_t cb, int32_t j, int p, T sc) {
      const int32_t a = cb - (cb / NN) * NN;
      double lv[BS];
#pragma unroll
      for (int cc = 0; cc < BS; cc++) lv[cc] = 0.0;
      if (b < NN) {
        const T* kr = s_ref + (size_t)(a * NN + b) * KB;
        if (j > 0) {
#pragma unroll
          for (int e = 0; e < KB; e++) acc[p * KB + e] += sc * kr[e];
        } else if (LIFT && j < 0) {
#pragma unroll
          for (int cc = 0; cc < BS; cc++)
#pragma unroll
            for (int dd = 0; dd < BS; dd++)
              lv[cc] += (double)(sc * kr[cc * BS + dd]) * __ldg(xd + (int64_t)(-j - 1) * BS + dd);
        }
      }
      if constexpr (LIFT) {
#pragma unroll
        for (int cc = 0; cc < BS; cc++) {
#pragma unroll
          for (int o = G >> 1; o; o >>= 1) lv[cc] += __shfl_xor_sync(gmask, lv[cc], o);
          if (gl == 0) bsum[cc] -= lv[cc];
        }
      }
      __syncwarp(gmask);
    };
    // the prefetched incidences (indices known at compile time), then the
    // rest -- a node in more than PF cells, none on a structured mesh -- in
    // a loop of their own, so that their FP64 scale computation stays out
    // of the common path
#pragma unroll
    for (int k = 0; k < PF; k++)
      if (k < nin) contribute(cbk[k], jk[k], pk[k], sck[k]);
    for (int k = PF; k < nin; k++) {
      const int32_t cb = __ldg(inc + ib + k);
      const int32_t c = cb / NN;
      const int32_t j = b < NN ? __ldg(cnd + (int64_t)c * NN + b) : 0;
      const int p = j > 0 ? find_col(cols, L, j - 1) : -1;
      contribute(cb, j, p, (T)(adet * (coef ? __ldg(coef + c) : 1.0)));
    }
    const int64_t ob = rb * KB;
    for (int i = gl; i < L * KB; i += G) {
      const T v = acc[i];
      if (v64) v64[ob + i] = (double)v;
      if (v32) v32[ob + i] = (float)v;
    }
    if (vec)
#pragma unroll
      for (int cc = 0; cc < BS; cc++) bvec[r * BS + cc] = bsum[cc];
    __syncwarp(gmask);  // the row slot is reused by the group's next row
  }
}

// launches k_kref + k_scatter_uniform; GT_ERR_UNSUPPORTED (nothing
// launched) when the reference block and the row slots do not fit in
// shared memory
template <int D, int ORDER, int BS, int FORM, class T>
static int launch_uniform(Matrix* A, const double* gref, const double* coef, double nu, const double* be,
                          double* bvec, const double* xd) {
  const Space* sp = A->space;
  Ctx* ctx = ctx_of(sp);
  constexpr int M1 = ORDER + 1;
  constexpr int NN = D == 2 ? M1 * M1 : M1 * M1 * M1;
  constexpr int G = NN <= 4 ? 4 : (NN <= 8 ? 8 : (NN <= 16 ? 16 : 32));
  constexpr int RPW = 32 / G;
  constexpr int KREF_N = NN * NN * BS * BS;
  constexpr size_t KREF_BYTES = ((size_t)KREF_N * sizeof(T) + 15) & ~size_t(15);
  int lmax = (A->max_row > 0 ? A->max_row : 1) | 1;  // odd slot stride (banks)
  double* v64 = A->precision != GT_FP32 ? A->val64 : nullptr;
  float* v32 = A->precision != GT_FP64 ? A->val32 : nullptr;
  // up to 16 warps per CTA where the row slots fit beside the reference
  // block (the loop is latency-bound: warps per SM decide its rate)
  int warps = 16;
  size_t per_row = (size_t)lmax * (BS * BS * sizeof(T) + sizeof(int32_t));
  while (warps > 1 && KREF_BYTES + (size_t)warps * RPW * per_row > 210 * 1024) warps >>= 1;
  size_t smem = KREF_BYTES + (size_t)warps * RPW * per_row;
  if (smem > 210 * 1024) return GT_ERR_UNSUPPORTED;
  auto kern = (be != nullptr && xd != nullptr) ? k_scatter_uniform<D, ORDER, BS, G, T, true>
                                               : k_scatter_uniform<D, ORDER, BS, G, T, false>;
  GT_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  GT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, smem));
  if (per_sm < 1) return GT_ERR_UNSUPPORTED;
  T* kref = nullptr;
  GT_TRY(dalloc(ctx, &kref, KREF_N));
  matrix_values_changed(A);
  T lamf = (T)(nu / ((1.0 + nu) * (1.0 - 2.0 * nu))), muf = (T)(1.0 / (2.0 * (1.0 + nu)));
  k_kref<D, ORDER, BS, FORM, T><<<GT_KC(ctx, (NN * NN + 127) / 128), 128, 0, ctx->stream>>>(gref, lamf, muf, kref);
  GT_LAUNCH(ctx, "k_kref");
  const int64_t rows_per_block = (int64_t)warps * RPW;
  const int64_t nblk = (A->nbrows + rows_per_block - 1) / rows_per_block;
  const int64_t cap = (int64_t)per_sm * ctx->num_sms;
  const int grid = (int)std::max<int64_t>(1, std::min(nblk, cap));
  kern<<<GT_KC(ctx, grid), warps * 32, smem, ctx->stream>>>(A->rowptr, A->colind, A->inc_ptr, A->inc, sp->cell_ndofs,
                                                             A->nbrows, lmax, kref, gref, coef, v64, v32, be, bvec, xd);
  cudaError_t e = cudaGetLastError();
  dfree(ctx, kref);  // stream-ordered: the pool hands the block out again only to later work
  if (e != cudaSuccess) return check_cuda(ctx, e, "k_scatter_uniform");
  return GT_OK;
}

template <int D, int ORDER, class T>
static int dispatch_uniform(Matrix* A, int form, const double* gref, const double* coef, double nu, const double* be,
                            double* bvec, const double* xd) {
  if (A->bs == 1) {
    if (form == GT_LAPLACE) return launch_uniform<D, ORDER, 1, GT_LAPLACE, T>(A, gref, coef, nu, be, bvec, xd);
    if (form == GT_MASS) return launch_uniform<D, ORDER, 1, GT_MASS, T>(A, gref, coef, nu, be, bvec, xd);
  } else {
    if (form == GT_LAPLACE) return launch_uniform<D, ORDER, D, GT_LAPLACE, T>(A, gref, coef, nu, be, bvec, xd);
    if (form == GT_MASS) return launch_uniform<D, ORDER, D, GT_MASS, T>(A, gref, coef, nu, be, bvec, xd);
    if (form == GT_ELASTICITY) return launch_uniform<D, ORDER, D, GT_ELASTICITY, T>(A, gref, coef, nu, be, bvec, xd);
  }
  return set_error(ctx_of(A->space), GT_ERR_UNSUPPORTED, "weak form not supported on this space");
}

template <int D, int ORDER, int BS, int FORM, class T>
static int launch_kron(Matrix* A, const T* Gc, double nu, const double* be, double* bvec, const double* xd) {
  const Space* sp = A->space;
  Ctx* ctx = ctx_of(sp);
  constexpr int M1 = ORDER + 1;
  constexpr int NN = D == 2 ? M1 * M1 : M1 * M1 * M1;
  constexpr int G = NN <= 4 ? 4 : (NN <= 8 ? 8 : (NN <= 16 ? 16 : 32));
  constexpr int RPW = 32 / G;
  int lmax = (A->max_row > 0 ? A->max_row : 1) | 1;  // odd slot stride (banks)
  matrix_values_changed(A);
  double* v64 = A->precision != GT_FP32 ? A->val64 : nullptr;
  float* v32 = A->precision != GT_FP64 ? A->val32 : nullptr;
  int warps = 4;
  size_t per_row = (size_t)lmax * (BS * BS * sizeof(T) + sizeof(int32_t));
  while (warps > 1 && (size_t)warps * RPW * per_row > 96 * 1024) warps >>= 1;
  size_t smem = (size_t)warps * RPW * per_row;
  if (smem > 200 * 1024) return set_error(ctx, GT_ERR_UNSUPPORTED, "sparsity row too wide for the scatter kernel");
  auto kern = k_scatter_kron<D, ORDER, BS, FORM, G, T, T>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int64_t rows_per_block = (int64_t)warps * RPW;
  int64_t grid = (A->nbrows + rows_per_block - 1) / rows_per_block;
  T lamf = (T)(nu / ((1.0 + nu) * (1.0 - 2.0 * nu))), muf = (T)(1.0 / (2.0 * (1.0 + nu)));
  kern<<<GT_KC(ctx, (unsigned)(grid > 0 ? grid : 1)), warps * 32, smem, ctx->stream>>>(
      A->rowptr, A->colind, A->inc_ptr, A->inc, sp->cell_ndofs, A->nbrows, lmax, Gc, lamf, muf, v64, v32, be, bvec, xd);
  GT_LAUNCH(ctx, "k_scatter_kron");
  return GT_OK;
}

template <int D, int ORDER, class T>
static int dispatch_kron(Matrix* A, int form, const T* Gc, double nu, const double* be, double* bvec,
                         const double* xd) {
  int bs = A->bs;
  if (bs == 1) {
    if (form == GT_LAPLACE) return launch_kron<D, ORDER, 1, GT_LAPLACE, T>(A, Gc, nu, be, bvec, xd);
    if (form == GT_MASS) return launch_kron<D, ORDER, 1, GT_MASS, T>(A, Gc, nu, be, bvec, xd);
  } else {
    if (form == GT_LAPLACE) return launch_kron<D, ORDER, D, GT_LAPLACE, T>(A, Gc, nu, be, bvec, xd);
    if (form == GT_MASS) return launch_kron<D, ORDER, D, GT_MASS, T>(A, Gc, nu, be, bvec, xd);
    if (form == GT_ELASTICITY) return launch_kron<D, ORDER, D, GT_ELASTICITY, T>(A, Gc, nu, be, bvec, xd);
  }
  return set_error(ctx_of(A->space), GT_ERR_UNSUPPORTED, "weak form not supported on this space");
}

static int alloc_values(Matrix* A);

// Sum-factorised numeric phase on affine QUAD4/HEX8 meshes.  Sets *used = 0
// (and writes only the load vector) when some cell is not affine.
static int kron_numeric(Matrix* A, int form, const double* coef, double nu, const double* f, const double* scoef,
                        double* be, double* bvec, const double* xd, int* used) {
  const Space* sp = A->space;
  Ctx* ctx = ctx_of(sp);
  *used = 0;
  int ct = sp->mesh->ctype;
  if (ct != GT_QUAD4 && ct != GT_HEX8) return GT_OK;
  if (form == GT_ELASTICITY && sp->ncomp != sp->mesh->D)
    return set_error(ctx, GT_ERR_UNSUPPORTED, "linear elasticity needs a vector space (tensor_size = (D,))");
  int64_t nc = sp->mesh->ncells;
  bool g64 = A->precision != GT_FP32;
  void* Gc = nullptr;
  uint32_t* flag = nullptr;
  double* gref = nullptr;
  GT_TRY(dalloc(ctx, (unsigned char**)&Gc, nc * GSTRIDE * (int64_t)(g64 ? sizeof(double) : sizeof(float))));
  GT_TRY(dalloc(ctx, &flag, 2));
  GT_TRY(dalloc(ctx, &gref, GSTRIDE));
  GT_CUDA(ctx, cudaMemsetAsync(flag, 0, 2 * sizeof(uint32_t), ctx->stream));
  double* gr = ctx->uniform_geom ? gref : nullptr;
  if (ct == GT_QUAD4) {
    if (gr) k_geom_ref<2, 4><<<GT_KC(ctx, 1), 32, 0, ctx->stream>>>(sp->mesh->coords, sp->mesh->cell_nodes, form, gr);
    k_geom_affine<2, 4><<<GT_KC(ctx, grid_for(nc, 256)), 256, 0, ctx->stream>>>(
        sp->mesh->coords, sp->mesh->cell_nodes, coef, form, sp->order, nc, sp->nn, sp->ncomp, Gc, g64, be, f, scoef,
        flag, ctx->d_err, gr, flag + 1);
  } else {
    if (gr) k_geom_ref<3, 8><<<GT_KC(ctx, 1), 32, 0, ctx->stream>>>(sp->mesh->coords, sp->mesh->cell_nodes, form, gr);
    k_geom_affine<3, 8><<<GT_KC(ctx, grid_for(nc, 256)), 256, 0, ctx->stream>>>(
        sp->mesh->coords, sp->mesh->cell_nodes, coef, form, sp->order, nc, sp->nn, sp->ncomp, Gc, g64, be, f, scoef,
        flag, ctx->d_err, gr, flag + 1);
  }
  GT_LAUNCH(ctx, "k_geom_affine");
  GT_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scratch[2], flag, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  GT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  uint32_t flags[2] = {0, 0};
  memcpy(flags, &ctx->h_scratch[2], 2 * sizeof(uint32_t));
  const uint32_t nonaffine = flags[0];
  const bool uniform = gr && !flags[1];
  mark(ctx, "elements");
  int s = GT_OK;
  if (!nonaffine) {
    s = alloc_values(A);
    int D = sp->mesh->D, o = sp->order;
    int us = GT_ERR_UNSUPPORTED;  // uniform path taken: GT_OK
    if (s == GT_OK && uniform) {
      us = g64 ? (D == 2 ? (o == 1 ? dispatch_uniform<2, 1, double>(A, form, gr, coef, nu, be, bvec, xd)
                                   : dispatch_uniform<2, 2, double>(A, form, gr, coef, nu, be, bvec, xd))
                         : (o == 1 ? dispatch_uniform<3, 1, double>(A, form, gr, coef, nu, be, bvec, xd)
                                   : dispatch_uniform<3, 2, double>(A, form, gr, coef, nu, be, bvec, xd)))
               : (D == 2 ? (o == 1 ? dispatch_uniform<2, 1, float>(A, form, gr, coef, nu, be, bvec, xd)
                                   : dispatch_uniform<2, 2, float>(A, form, gr, coef, nu, be, bvec, xd))
                         : (o == 1 ? dispatch_uniform<3, 1, float>(A, form, gr, coef, nu, be, bvec, xd)
                                   : dispatch_uniform<3, 2, float>(A, form, gr, coef, nu, be, bvec, xd)));
      if (us != GT_OK && us != GT_ERR_UNSUPPORTED) s = us;
    }
    if (s == GT_OK && us == GT_ERR_UNSUPPORTED) {
      if (g64) {
        const double* G = (const double*)Gc;
        s = D == 2 ? (o == 1 ? dispatch_kron<2, 1, double>(A, form, G, nu, be, bvec, xd)
                             : dispatch_kron<2, 2, double>(A, form, G, nu, be, bvec, xd))
                   : (o == 1 ? dispatch_kron<3, 1, double>(A, form, G, nu, be, bvec, xd)
                             : dispatch_kron<3, 2, double>(A, form, G, nu, be, bvec, xd));
      } else {
        const float* G = (const float*)Gc;
        s = D == 2 ? (o == 1 ? dispatch_kron<2, 1, float>(A, form, G, nu, be, bvec, xd)
                             : dispatch_kron<2, 2, float>(A, form, G, nu, be, bvec, xd))
                   : (o == 1 ? dispatch_kron<3, 1, float>(A, form, G, nu, be, bvec, xd)
                             : dispatch_kron<3, 2, float>(A, form, G, nu, be, bvec, xd));
      }
    }
    mark(ctx, "scatter");
    if (s == GT_OK) *used = 1;
  }
  pool_free(ctx, Gc);
  dfree(ctx, flag);
  dfree(ctx, gref);
  return s;
}

// vector scatter: each (row, component) sums its cells in the order of
// row_load_sum
__global__ void k_scatter_vec(const int64_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc, int nn, int bs,
                              int64_t nrows, const double* __restrict__ be, double* __restrict__ b) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nrows * bs) return;
  int64_t r = t / bs;
  int k = (int)(t - r * bs);
  // the order of row_load_sum, one thread per (row, component)
  const int64_t ib = inc_ptr[r], ie = inc_ptr[r + 1];
  double s[4];
#pragma unroll
  for (int j = 0; j < 4; j++) load_partial<1>(ib, ie, j, inc, nn, bs, be + k, &s[j]);
  b[t] = (s[0] + s[1]) + (s[2] + s[3]);
}

int scatter_vector(const Space* sp, const int64_t* inc_ptr, const int32_t* inc, const double* be, double* b) {
  Ctx* ctx = ctx_of(sp);
  int64_t n = sp->nfree_nodes * sp->ncomp;
  k_scatter_vec<<<GT_KC(ctx, grid_for(n, 256)), 256, 0, ctx->stream>>>(inc_ptr, inc, sp->nn, sp->ncomp, sp->nfree_nodes, be, b);
  GT_LAUNCH(ctx, "k_scatter_vec");
  return GT_OK;
}

__global__ void k_find_diag(const int64_t* rowptr, const int32_t* colind, int64_t n, int32_t* pos, uint32_t* err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  int64_t b = rowptr[r], e = rowptr[r + 1];
  int32_t p = -1;
  int64_t lo = b, hi = e - 1;
  while (lo <= hi) {
    int64_t mid = (lo + hi) >> 1;
    int32_t c = colind[mid];
    if (c == r) { p = (int32_t)(mid - b); break; }
    if (c < r) lo = mid + 1; else hi = mid - 1;
  }
  if (p < 0) atomicOr(err, DEV_ERR_LOOKUP);
  pos[r] = p < 0 ? 0 : p;
}

int find_diag(Matrix* A) {
  Ctx* ctx = ctx_of(A->space);
  if (A->diag_pos) return GT_OK;
  GT_TRY(dalloc(ctx, &A->diag_pos, A->nbrows + 1));
  k_find_diag<<<GT_KC(ctx, grid_for(A->nbrows, 256)), 256, 0, ctx->stream>>>(A->rowptr, A->colind, A->nbrows, A->diag_pos, ctx->d_err);
  GT_LAUNCH(ctx, "k_find_diag");
  return GT_OK;
}

// scalar CSR expansion of a block CSR matrix (download path)
__global__ void k_expand_rowptr(const int64_t* rowptr, int64_t nbrows, int bs, int64_t* out) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t > nbrows * bs) return;
  if (t == nbrows * bs) { out[t] = rowptr[nbrows] * bs * bs; return; }
  int64_t i = t / bs;
  int c = (int)(t - i * bs);
  int64_t len = rowptr[i + 1] - rowptr[i];
  out[t] = rowptr[i] * bs * bs + (int64_t)c * bs * len;
}
template <class V>
__global__ void k_expand_entries(const int64_t* rowptr, const int32_t* colind, const V* vals, int64_t nbrows, int bs,
                                 int32_t* ocol, V* oval) {
  int64_t i = blockIdx.x;  // block row
  if (i >= nbrows) return;
  int64_t b = rowptr[i];
  int64_t len = rowptr[i + 1] - b;
  for (int64_t t = threadIdx.x; t < len * bs * bs; t += blockDim.x) {
    int64_t c = t / (len * bs);
    int64_t r = t - c * len * bs;
    int64_t k = r / bs;
    int d = (int)(r - k * bs);
    int64_t o = b * bs * bs + t;
    if (ocol) ocol[o] = colind[b + k] * bs + d;
    if (oval) oval[o] = vals[(b + k) * bs * bs + c * bs + d];
  }
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
// a pointer the kernels can read: device pointers pass through, host data is
// staged into a pooled device buffer
// With async, a host source is uploaded on the copy stream and wait()
// orders the main stream after it (the upload overlaps the kernels queued
// before the consumer).
template <class T>
struct DevIn {
  Ctx* ctx = nullptr;
  const T* p = nullptr;
  T* owned = nullptr;
  cudaEvent_t ev = nullptr;
  int init(Ctx* c, const T* src, int64_t n, bool async = false) {
    ctx = c;
    if (!src) return GT_OK;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, src) == cudaSuccess &&
        (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged)) {
      if (at.type == cudaMemoryTypeDevice && at.device != c->device)
        return set_error(c, GT_ERR_INVALID, "input array is memory of another device");
      p = src;
      return GT_OK;
    }
    cudaGetLastError();
    GT_TRY(dalloc(c, &owned, n));
    if (async) GT_TRY(side_copy_in(c, owned, src, sizeof(T) * (size_t)n, &ev));
    else GT_TRY(copy_in(c, owned, src, n));
    p = owned;
    return GT_OK;
  }
  void wait() {
    if (ev) {
      cudaStreamWaitEvent(ctx->stream, ev, 0);
      event_put(ctx, ev);
      ev = nullptr;
    }
  }
  // orders stream s after the upload (which stays pending for the main stream)
  void wait_on(cudaStream_t s) const {
    if (ev) cudaStreamWaitEvent(s, ev, 0);
  }
  ~DevIn() {
    wait();
    if (owned) dfree(ctx, owned);
  }
};

// the per-call inputs of the numeric phase (per-cell coefficient, source,
// source coefficient, Dirichlet values), staged before the sparsity phase
struct NumIn {
  DevIn<double> coef, f, scoef, xd;
  int init(const Space* sp, const double* coef_in, const double* f_in, const double* scoef_in, const double* xd_in,
           bool async) {
    Ctx* ctx = sp->mesh->ctx;
    int64_t nc = sp->mesh->ncells;
    GT_TRY(coef.init(ctx, coef_in, nc, async));
    GT_TRY(f.init(ctx, f_in, sp->ncomp, async));
    GT_TRY(scoef.init(ctx, scoef_in, nc, async));
    GT_TRY(xd.init(ctx, xd_in, sp->ndiri_nodes * sp->ncomp, async));
    return GT_OK;
  }
  void wait() {
    coef.wait();
    f.wait();
    scoef.wait();
    xd.wait();
  }
  void wait_on(cudaStream_t s) const {
    coef.wait_on(s);
    f.wait_on(s);
    scoef.wait_on(s);
    xd.wait_on(s);
  }
};

// Element matrices (and vectors) launched on the auxiliary compute stream
// before the sparsity kernels; numeric_in joins the streams before the
// scatter.  The auxiliary stream has the lowest priority, so its blocks fill
// the SMs the sparsity kernels leave idle (their host round trips, their
// tails) rather than run beside them: measured on GB300, FP64-bound blocks
// co-resident with the sparsity kernels slow those 2.5x (an FP64 warp
// instruction holds its SM sub-partition's dispatch for many cycles), while
// the sparsity result is what the host downloads first.  Taken for the cells
// without the factored (Kronecker) path -- tetrahedra -- and not while phases
// are being timed (the phase marks time each kernel alone).  All of the
// stage's device blocks are held until the join: a block freed earlier could
// be handed to main-stream work while the auxiliary kernels still use it.
struct EarlyElems {
  bool active = false;
  void* Ke = nullptr;
  double* be = nullptr;
  double* tab = nullptr;
  cudaEvent_t done = nullptr;
  ElemChunks chunks;  // chunked launches (P1): the event of each cell chunk
};

static void early_put_chunk_events(Ctx* ctx, EarlyElems* E) {
  for (int i = 0; i < kRowChunks; i++)
    if (E->chunks.ev[i]) event_put(ctx, E->chunks.ev[i]);
  E->chunks = ElemChunks{};
}

static int elements_early(const Space* sp, int form, const NumIn& in, double nu, int precision, bool want_b,
                          bool chunked, EarlyElems* E) {
  Ctx* ctx = ctx_of(sp);
  if (ctx->prof || !ctx->overlap || !ctx->aux || sp->mesh->ctype != GT_TET4) return GT_OK;
  // only when the main stream outranks the auxiliary one (the context's own
  // stream does; a caller's stream of default priority does not -- then the
  // element blocks would hold the SMs ahead of the sparsity kernels)
  int pm = 0, pa = 0;
  if (cudaStreamGetPriority(ctx->stream, &pm) != cudaSuccess || cudaStreamGetPriority(ctx->aux, &pa) != cudaSuccess) {
    cudaGetLastError();
    return GT_OK;
  }
  if (!(pm < pa)) return GT_OK;
  if (form != GT_LAPLACE && form != GT_MASS && form != GT_ELASTICITY) return GT_OK;  // reported by numeric_in
  const int64_t nc = sp->mesh->ncells;
  const int kprec = precision == GT_FP32 ? GT_FP32 : GT_FP64;
  const size_t esz = kprec == GT_FP32 ? sizeof(float) : sizeof(double);
  cudaEvent_t start = event_get(ctx);
  E->done = event_get(ctx);
  if (!start || !E->done) return set_error(ctx, GT_ERR_CUDA, "cudaEventCreate failed");
  E->chunks.n = chunked ? kRowChunks : 0;
  for (int i = 0; i < E->chunks.n; i++) {
    E->chunks.ev[i] = event_get(ctx);
    if (!E->chunks.ev[i]) {
      event_put(ctx, start);
      event_put(ctx, E->done);
      early_put_chunk_events(ctx, E);
      *E = EarlyElems{};
      return set_error(ctx, GT_ERR_CUDA, "cudaEventCreate failed");
    }
  }
  // the auxiliary stream starts after all work queued so far (mesh, space,
  // and every block the pool may hand out below) and after the uploads
  GT_CUDA(ctx, cudaEventRecord(start, ctx->stream));
  GT_CUDA(ctx, cudaStreamWaitEvent(ctx->aux, start, 0));
  event_put(ctx, start);
  in.wait_on(ctx->aux);
  mesh_wait_coords_on(sp->mesh, ctx->aux);
  if (want_b) GT_TRY(dalloc(ctx, &E->be, nc * sp->nloc));
  GT_TRY(dalloc(ctx, (unsigned char**)&E->Ke, (int64_t)(nc * ke_per_cell(sp) * esz)));
  cudaStream_t main_stream = ctx->stream;
  ctx->stream = ctx->aux;
  int s = compute_elements(sp, form, in.coef.p, nu, precision, in.f.p, in.scoef.p, E->Ke, E->be, 1, &E->tab,
                           chunked ? &E->chunks : nullptr);
  if (s == GT_OK && cudaEventRecord(E->done, ctx->aux) != cudaSuccess) s = check_cuda(ctx, cudaGetLastError(), "event");
  ctx->stream = main_stream;
  if (s != GT_OK) {
    // nothing of the stage may be reused before the auxiliary stream drains
    cudaStreamSynchronize(ctx->aux);
    if (E->tab) dfree(ctx, E->tab);
    if (E->Ke) pool_free(ctx, E->Ke);
    if (E->be) dfree(ctx, E->be);
    event_put(ctx, E->done);
    early_put_chunk_events(ctx, E);
    *E = EarlyElems{};
    return s;
  }
  E->active = true;
  return GT_OK;
}

// the main stream waits for the whole element stage; its events and its
// tabulation block go back to the context
static int join_stage(Ctx* ctx, EarlyElems* E) {
  if (!E->active) return GT_OK;
  E->active = false;
  cudaError_t e = cudaStreamWaitEvent(ctx->stream, E->done, 0);
  event_put(ctx, E->done);
  E->done = nullptr;
  early_put_chunk_events(ctx, E);
  if (e != cudaSuccess) {
    cudaStreamSynchronize(ctx->aux);
    dfree(ctx, E->tab);
    return check_cuda(ctx, e, "join of the element stage");
  }
  dfree(ctx, E->tab);  // later users of the block are ordered after the join
  return GT_OK;
}

// releases a stage that numeric_in did not take over (error paths)
static void early_release(Ctx* ctx, EarlyElems* E) {
  if (!E->active) return;
  cudaStreamSynchronize(ctx->aux);
  dfree(ctx, E->tab);
  pool_free(ctx, E->Ke);
  if (E->be) dfree(ctx, E->be);
  event_put(ctx, E->done);
  early_put_chunk_events(ctx, E);
  *E = EarlyElems{};
}

static bool is_device_ptr(const void* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

static int alloc_values(Matrix* A) {
  Ctx* ctx = ctx_of(A->space);
  int64_t nv = A->bnnz * A->bs * A->bs;
  if (A->precision != GT_FP32 && !A->val64) GT_TRY(dalloc(ctx, &A->val64, nv));
  if (A->precision != GT_FP64 && !A->val32) GT_TRY(dalloc(ctx, &A->val32, nv));
  return GT_OK;
}

// host CSR outputs filled by the assembly call itself (scalar entries)
struct HostCsr {
  int64_t* rowptr;
  int32_t* colind;
  double* v64;
  float* v32;
  int64_t capacity;  // entries colind / values can hold
};

// element matrices + scatter on the existing pattern (and optionally b).
// in.xd (optional, with b_out): Dirichlet values, ndiri_nodes * ncomp in the
// Dirichlet numbering; b_out then receives b - Ad xd (src/problems.jl:439-453).
// hc (optional, scalar matrices): host CSR outputs whose pattern is being
// downloaded on the copy stream (pat_down: its event); the values are then
// scattered in row chunks, each chunk's download overlapping the next chunk's
// scatter (*values_done set when that happened).
static int numeric_pass(Matrix* A, int form, NumIn& in, double nu, double* b_out, const HostCsr* hc,
                        cudaEvent_t pat_down, bool* values_done, EarlyElems* early) {
  const Space* sp = A->space;
  Ctx* ctx = ctx_of(sp);
  int64_t nc = sp->mesh->ncells;
  in.wait();
  mesh_wait_coords(sp->mesh);
  DevIn<double>&coef = in.coef, &f = in.f, &scoef = in.scoef, &xd = in.xd;
  int kprec = A->precision == GT_FP32 ? GT_FP32 : GT_FP64;
  size_t esz = kprec == GT_FP32 ? sizeof(float) : sizeof(double);
  void* Ke = nullptr;
  double* be = nullptr;
  const bool pre = early && early->active;
  bool b_copied = false;  // a host b already downloaded chunk by chunk
  // element stage already queued on the auxiliary stream: taken over here.
  // When the values go to host buffers chunk by chunk and the stage was
  // launched in cell chunks (P1), it is pipelined with the scatter: each row
  // chunk's scatter waits only for the element chunks up to its rows' last
  // cell, so the downloads start while elements are still computed, and the
  // whole stage is joined after the last chunk.  Otherwise it is joined
  // before the scatter (on device buffers that is faster: scatter blocks
  // beside FP64-bound element blocks run slower than after them)
  EarlyElems stage;
  const bool host_chunks = hc && pat_down && A->bs == 1 && values_done;
  const bool piped = host_chunks && pre && early->chunks.n == kRowChunks && A->chunk_last_ok;
  if (pre) {
    stage = *early;
    *early = EarlyElems{};
    Ke = stage.Ke;
    be = stage.be;
    if (!piped) GT_TRY(join_stage(ctx, &stage));
  } else if (b_out) {
    GT_TRY(dalloc(ctx, &be, nc * sp->nloc));
  }
  // the main stream waits for the element chunks that hold row chunk k's cells
  auto wait_rows = [&](int k) -> int {
    const int32_t last = A->chunk_last[k];
    int j = 0;
    while (j < stage.chunks.n - 1 && stage.chunks.end[j] <= last) j++;
    GT_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, stage.chunks.ev[j], 0));
    return GT_OK;
  };
  const bool dev = b_out && is_device_ptr(b_out);
  double* bd = b_out;
  const int64_t nb = sp->nfree_nodes * sp->ncomp;
  int s = GT_OK;
  if (b_out && !dev) s = dalloc(ctx, &bd, nb);  // errors fall through to the stage release below
  int used_kron = 0;
  // the load vector (and the Dirichlet lift) is summed inside the matrix
  // scatter, over the same incidences
  if (s == GT_OK && !pre)
    s = kron_numeric(A, form, coef.p, nu, f.p, scoef.p, be, b_out ? bd : nullptr, b_out ? xd.p : nullptr, &used_kron);
  if (s == GT_OK && !used_kron) {
    if (!pre) {
      s = dalloc(ctx, (unsigned char**)&Ke, (int64_t)(nc * ke_per_cell(sp) * esz));
      if (s == GT_OK) s = compute_elements(sp, form, coef.p, nu, A->precision, f.p, scoef.p, Ke, be, 1);
    }
    mark(ctx, "elements");
    if (s == GT_OK) s = alloc_values(A);
    if (s == GT_OK && host_chunks) {
      // all chunks are queued first (the device never waits for the host),
      // then the host row pointers -- downloaded meanwhile -- give each
      // chunk's range for its download behind the chunk's event; a host b
      // comes back chunk by chunk too, so only the last chunk's rows are left
      // to copy after the last scatter
      constexpr int NCH = kRowChunks;
      cudaEvent_t evs[NCH] = {};
      int nq = 0;
      for (int k = 0; k < NCH && s == GT_OK; k++, nq++) {
        const int64_t r0 = A->nbrows * k / NCH, r1 = A->nbrows * (k + 1) / NCH;
        if (piped) s = wait_rows(k);
        if (s == GT_OK)
          s = scatter_matrix(A, Ke, kprec, A->precision, be, b_out ? bd : nullptr, b_out ? xd.p : nullptr, r0, r1);
        evs[k] = event_get(ctx);
        if (s == GT_OK && !evs[k]) s = set_error(ctx, GT_ERR_CUDA, "cudaEventCreate failed");
        if (s == GT_OK && cudaEventRecord(evs[k], ctx->stream) != cudaSuccess)
          s = check_cuda(ctx, cudaGetLastError(), "event");
      }
      if (s == GT_OK) {
        cudaError_t e = cudaEventSynchronize(pat_down);
        if (e != cudaSuccess) s = check_cuda(ctx, e, "pattern download");
      }
      const bool b_side = b_out && !dev;
      for (int k = 0; k < NCH && s == GT_OK; k++) {
        const int64_t r0 = A->nbrows * k / NCH, r1 = A->nbrows * (k + 1) / NCH;
        const int64_t o0 = hc->rowptr[r0], o1 = hc->rowptr[r1];
        cudaStreamWaitEvent(ctx->side, evs[k], 0);
        if (o1 > o0 && hc->v64 && A->val64)
          cudaMemcpyAsync(hc->v64 + o0, A->val64 + o0, sizeof(double) * (o1 - o0), cudaMemcpyDefault, ctx->side);
        if (o1 > o0 && hc->v32 && A->val32)
          cudaMemcpyAsync(hc->v32 + o0, A->val32 + o0, sizeof(float) * (o1 - o0), cudaMemcpyDefault, ctx->side);
        if (b_side && r1 > r0)  // scalar rows: b entries r0..r1
          cudaMemcpyAsync(b_out + r0, bd + r0, sizeof(double) * (r1 - r0), cudaMemcpyDefault, ctx->side);
        cudaError_t ce = cudaGetLastError();
        if (ce != cudaSuccess) s = check_cuda(ctx, ce, "values download");
      }
      for (int k = 0; k < nq; k++)
        if (evs[k]) event_put(ctx, evs[k]);
      if (s == GT_OK && b_side) {
        // the staging block of b is freed below: later main-stream users of
        // the block wait for the copies out of it
        cudaEvent_t bev = event_get(ctx);
        if (!bev) {
          s = set_error(ctx, GT_ERR_CUDA, "cudaEventCreate failed");
        } else {
          cudaEventRecord(bev, ctx->side);
          cudaStreamWaitEvent(ctx->stream, bev, 0);
          event_put(ctx, bev);
          b_copied = true;
        }
      }
      if (s == GT_OK) *values_done = true;
    } else if (s == GT_OK) {
      s = scatter_matrix(A, Ke, kprec, A->precision, be, b_out ? bd : nullptr, b_out ? xd.p : nullptr);
    }
    mark(ctx, "scatter");
  }
  if (stage.active) {
    if (s == GT_OK) {
      s = join_stage(ctx, &stage);
    } else {
      // nothing of the stage may be reused before the auxiliary stream drains
      cudaStreamSynchronize(ctx->aux);
      event_put(ctx, stage.done);
      early_put_chunk_events(ctx, &stage);
      dfree(ctx, stage.tab);
      stage.active = false;
    }
  }
  // host b: the copy is queued here; the caller's device_status() call
  // synchronises the stream before returning (the freed staging block is only
  // reused by work queued after the copy)
  if (s == GT_OK && b_out && !dev && !b_copied) s = copy_out(ctx, b_out, bd, nb);
  if (b_out && !dev) dfree(ctx, bd);
  if (Ke) pool_free(ctx, Ke);
  if (be) dfree(ctx, be);
  return s;
}

// FP32 values of a GT_MIXED matrix integrated in FP32 (FP64 Jacobian, its
// inverse and determinant; FP32 element blocks and FP32 accumulation), on the
// pattern the FP64 pass built
static int fp32_values_pass(Matrix* A, int form, NumIn& in, double nu) {
  const Space* sp = A->space;
  Ctx* ctx = ctx_of(sp);
  int used = 0;
  GT_TRY(kron_numeric(A, form, in.coef.p, nu, nullptr, nullptr, nullptr, nullptr, nullptr, &used));
  if (used) return GT_OK;
  void* Ke = nullptr;
  GT_TRY(dalloc(ctx, (unsigned char**)&Ke, (int64_t)(sp->mesh->ncells * ke_per_cell(sp) * sizeof(float))));
  int s = compute_elements(sp, form, in.coef.p, nu, GT_FP32, nullptr, nullptr, Ke, nullptr, 1);
  if (s == GT_OK) s = alloc_values(A);
  if (s == GT_OK) s = scatter_matrix(A, Ke, GT_FP32, GT_FP32, nullptr, nullptr, nullptr);
  pool_free(ctx, Ke);
  return s;
}

// element matrices + scatter on the existing pattern (and optionally b).  A
// GT_MIXED matrix takes two passes: FP64 integration into the FP64 values
// (and b), then FP32 integration into the FP32 values
static int numeric_in(Matrix* A, int form, NumIn& in, double nu, double* b_out, const HostCsr* hc = nullptr,
                      cudaEvent_t pat_down = nullptr, bool* values_done = nullptr, EarlyElems* early = nullptr) {
  if (A->precision != GT_MIXED) return numeric_pass(A, form, in, nu, b_out, hc, pat_down, values_done, early);
  A->precision = GT_FP64;
  int s = numeric_pass(A, form, in, nu, b_out, hc, pat_down, values_done, early);
  A->precision = GT_FP32;
  if (s == GT_OK) s = fp32_values_pass(A, form, in, nu);
  A->precision = GT_MIXED;
  if (s == GT_OK && hc && values_done && *values_done && hc->v32 && A->bs == 1 && A->bnnz > 0)
    s = copy_out(ctx_of(A->space), hc->v32, A->val32, A->bnnz);
  return s;
}

static int numeric(Matrix* A, int form, const double* coef_in, double nu, const double* f_in, const double* scoef_in,
                   double* b_out, const double* xd_in = nullptr) {
  NumIn in;
  GT_TRY(in.init(A->space, coef_in, f_in, scoef_in, b_out ? xd_in : nullptr, false));
  return numeric_in(A, form, in, nu, b_out);
}

static int device_status(Ctx* ctx, const char* where) {
  uint32_t bits = 0;
  GT_TRY(take_device_error(ctx, &bits));
  if (!bits) return GT_OK;
  if (bits & DEV_ERR_DEGENERATE) return set_error(ctx, GT_ERR_INVALID, std::string(where) + ": degenerate cell (det J = 0)");
  return set_error(ctx, GT_ERR_INVALID, std::string(where) + ": device-side check failed");
}

}  // namespace gt

using namespace gt;

static void matrix_release(gt_matrix* A) {
  Ctx* c = A->ctx;
  dfree(c, A->rowptr);
  dfree(c, A->colind);
  dfree(c, A->val64);
  dfree(c, A->val32);
  dfree(c, A->inc_ptr);
  dfree(c, A->inc);
  dfree(c, A->diag_pos);
  sell_release(A);
}

extern "C" {

static int assemble_mv(gt_space* sp, int form, const double* cell_coef, double nu, int precision, const double* f,
                       const double* source_coef, const double* xd, double* b, gt_matrix** out,
                       const HostCsr* hc = nullptr);

int gt_assemble_matrix_and_vector(gt_space* sp, int form, const double* cell_coef, double nu, int precision,
                                  const double* f, const double* source_coef, double* b, gt_matrix** out) {
  return assemble_mv(sp, form, cell_coef, nu, precision, f, source_coef, nullptr, b, out);
}

int gt_linear_problem(gt_space* sp, int form, const double* cell_coef, double nu, int precision, const double* f,
                      const double* source_coef, const double* dirichlet_values, double* b, gt_matrix** out) {
  if (!sp || !b || !f) return GT_ERR_INVALID;
  return assemble_mv(sp, form, cell_coef, nu, precision, f, source_coef, dirichlet_values, b, out);
}

int gt_assemble_csr(gt_space* sp, int form, const double* cell_coef, double nu, int precision, const double* f,
                    const double* source_coef, double* b, int64_t capacity, int64_t* rowptr, int32_t* colind,
                    double* values64, float* values32, gt_matrix** out) {
  if (!sp || !rowptr || !colind) return GT_ERR_INVALID;
  HostCsr hc{rowptr, colind, values64, values32, capacity};
  return assemble_mv(sp, form, cell_coef, nu, precision, f, source_coef, nullptr, b, out, &hc);
}

}  // extern "C"

static int assemble_mv(gt_space* sp, int form, const double* cell_coef, double nu, int precision, const double* f,
                       const double* source_coef, const double* xd, double* b, gt_matrix** out, const HostCsr* hc) {
  if (!sp || !out) return GT_ERR_INVALID;
  *out = nullptr;
  Ctx* ctx = sp->mesh->ctx;
  if (precision != GT_FP64 && precision != GT_FP32 && precision != GT_MIXED)
    return set_error(ctx, GT_ERR_INVALID, "precision must be GT_FP64, GT_FP32 or GT_MIXED");
  if (form != GT_LAPLACE && form != GT_MASS && form != GT_ELASTICITY)
    return set_error(ctx, GT_ERR_UNSUPPORTED, "weak form not supported (Laplacian, mass, linear elasticity only)");
  if (form == GT_ELASTICITY && sp->ncomp != sp->mesh->D)
    return set_error(ctx, GT_ERR_UNSUPPORTED, "linear elasticity needs a vector space (tensor_size = (D,))");
  if (b && !f) return set_error(ctx, GT_ERR_INVALID, "vector assembly needs a source f");
  cudaSetDevice(ctx->device);
  gt_matrix* A = new gt_matrix();
  A->ctx = ctx;
  A->space = sp;
  A->bs = sp->ncomp;
  A->precision = precision;
  mark(ctx, "setup");
  // host inputs upload on the copy stream while the sparsity is built
  NumIn in;
  int s = in.init(sp, cell_coef, f, source_coef, b ? xd : nullptr, true);
  // element kernels on the auxiliary stream, beside the sparsity kernels
  EarlyElems early;
  // (in cell chunks when the values go to host buffers: the scatter and the
  // downloads then start on the first chunks)
  if (s == GT_OK) s = elements_early(sp, form, in, nu, precision, b != nullptr, hc != nullptr, &early);
  // incidence + sparsity (+ each row chunk's last cell for the pipelined
  // scatter into host buffers)
  if (s == GT_OK) s = build_pattern(A, hc != nullptr);
  cudaEvent_t side_done = nullptr;
  const int bs = A->bs;
  const int64_t nscal = A->nbrows * bs, nnz = A->bnnz * bs * bs;
  if (s == GT_OK && hc && nnz > hc->capacity)
    s = set_error(ctx, GT_ERR_INVALID, "gt_assemble_csr: capacity " + std::to_string(hc->capacity) +
                                           " below the " + std::to_string(nnz) + " entries");
  if (s == GT_OK && hc && bs == 1) {
    // the pattern goes back to the host while the values are computed
    cudaEvent_t pat = event_get(ctx);
    side_done = event_get(ctx);
    if (!pat || !side_done) s = set_error(ctx, GT_ERR_CUDA, "cudaEventCreate failed");
    if (s == GT_OK && cudaEventRecord(pat, ctx->stream) != cudaSuccess) s = check_cuda(ctx, cudaGetLastError(), "event");
    if (s == GT_OK) cudaStreamWaitEvent(ctx->side, pat, 0);
    if (s == GT_OK && cudaMemcpyAsync(hc->rowptr, A->rowptr, sizeof(int64_t) * (nscal + 1), cudaMemcpyDefault,
                                      ctx->side) != cudaSuccess)
      s = check_cuda(ctx, cudaGetLastError(), "rowptr download");
    if (s == GT_OK && nnz > 0 &&
        cudaMemcpyAsync(hc->colind, A->colind, sizeof(int32_t) * nnz, cudaMemcpyDefault, ctx->side) != cudaSuccess)
      s = check_cuda(ctx, cudaGetLastError(), "colind download");
    if (s == GT_OK) cudaEventRecord(side_done, ctx->side);
    event_put(ctx, pat);
  }
  bool values_done = false;
  if (s == GT_OK) s = numeric_in(A, form, in, nu, b, hc, side_done, &values_done, &early);
  early_release(ctx, &early);  // error paths: a stage numeric_in did not take over
  if (s == GT_OK && hc && !values_done) {
    if (bs == 1) {
      if (hc->v64 && A->val64 && nnz > 0) s = copy_out(ctx, hc->v64, A->val64, nnz);
      if (s == GT_OK && hc->v32 && A->val32 && nnz > 0) s = copy_out(ctx, hc->v32, A->val32, nnz);
    } else {
      s = gt_matrix_download_csr(A, hc->rowptr, hc->colind, hc->v64, hc->v32);
    }
  }
  if (s == GT_OK) s = device_status(ctx, "assemble_matrix");  // synchronises the stream
  if (side_done) {
    cudaError_t e = cudaStreamSynchronize(ctx->side);  // pattern and chunked value downloads
    if (s == GT_OK && e != cudaSuccess) s = check_cuda(ctx, e, "host CSR download");
    event_put(ctx, side_done);
  }
  if (s != GT_OK) {
    cudaStreamSynchronize(ctx->side);
    matrix_release(A);
    delete A;
    return s;
  }
  *out = A;
  return GT_OK;
}

extern "C" {

int gt_assemble_matrix(gt_space* sp, int form, const double* cell_coef, double nu, int precision, gt_matrix** out) {
  return gt_assemble_matrix_and_vector(sp, form, cell_coef, nu, precision, nullptr, nullptr, nullptr, out);
}

int gt_update_matrix(gt_matrix* A, int form, const double* cell_coef, double nu) {
  if (!A) return GT_ERR_INVALID;
  Ctx* ctx = A->space->mesh->ctx;
  GT_TRY(numeric(A, form, cell_coef, nu, nullptr, nullptr, nullptr));
  return device_status(ctx, "update_matrix");
}

int gt_update_matrix_and_vector(gt_matrix* A, int form, const double* cell_coef, double nu, const double* f,
                                const double* source_coef, double* b) {
  if (!A) return GT_ERR_INVALID;
  Ctx* ctx = A->space->mesh->ctx;
  if (b && !f) return set_error(ctx, GT_ERR_INVALID, "vector assembly needs a source f");
  GT_TRY(numeric(A, form, cell_coef, nu, f, source_coef, b));
  return device_status(ctx, "update_matrix");
}

int gt_assemble_vector(gt_space* sp, const double* f, const double* cell_coef, double* b) {
  if (!sp || !f || !b) return GT_ERR_INVALID;
  Ctx* ctx = sp->mesh->ctx;
  cudaSetDevice(ctx->device);
  if (!sp->inc) GT_TRY(build_incidence(ctx, sp, &sp->inc_ptr, &sp->inc, &sp->ninc, true));
  int64_t nc = sp->mesh->ncells;
  DevIn<double> coef, fd;
  GT_TRY(coef.init(ctx, cell_coef, nc));
  GT_TRY(fd.init(ctx, f, sp->ncomp));
  double* be = nullptr;
  GT_TRY(dalloc(ctx, &be, nc * sp->nloc));
  mesh_wait_coords(sp->mesh);
  int s = compute_elements(sp, GT_MASS, nullptr, 0.0, GT_FP64, fd.p, coef.p, nullptr, be, 0);
  int64_t nb = sp->nfree_nodes * sp->ncomp;
  bool dev = is_device_ptr(b);
  double* bd = b;
  if (s == GT_OK && !dev) s = dalloc(ctx, &bd, nb);
  if (s == GT_OK) s = scatter_vector(sp, sp->inc_ptr, sp->inc, be, bd);
  if (s == GT_OK && !dev) s = copy_out(ctx, b, bd, nb);
  if (s == GT_OK) s = device_status(ctx, "assemble_vector");
  if (!dev && bd) dfree(ctx, bd);
  dfree(ctx, be);
  return s;
}

int gt_integrate(gt_space* sp, int kind, const double* u_free, const double* u_dirichlet, const double* poly,
                 double* result) {
  if (!sp || !result) return GT_ERR_INVALID;
  Ctx* ctx = sp->mesh->ctx;
  if (kind < GT_INT_VOLUME || kind > GT_INT_H1_ERROR2)
    return set_error(ctx, GT_ERR_INVALID, "gt_integrate: unknown integrand kind");
  const bool need_u = kind >= GT_INT_FIELD, need_p = kind == GT_INT_POLY || kind >= GT_INT_L2_ERROR2;
  if (need_u && !u_free) return set_error(ctx, GT_ERR_INVALID, "gt_integrate: this integrand needs u_free");
  if (need_p && !poly) return set_error(ctx, GT_ERR_INVALID, "gt_integrate: this integrand needs poly");
  cudaSetDevice(ctx->device);
  DevIn<double> uf, ud, pc;
  GT_TRY(uf.init(ctx, need_u ? u_free : nullptr, sp->nfree_nodes * sp->ncomp));
  GT_TRY(ud.init(ctx, need_u ? u_dirichlet : nullptr, sp->ndiri_nodes * sp->ncomp));
  GT_TRY(pc.init(ctx, need_p ? poly : nullptr, (int64_t)kPolyCoefs * (kind == GT_INT_POLY ? 1 : sp->ncomp)));
  double v = 0.0;
  int s = integrate(sp, kind, uf.p, ud.p, pc.p, &v);
  if (s == GT_OK) s = device_status(ctx, "integrate");
  if (s == GT_OK) *result = v;
  return s;
}

int gt_matrix_info(const gt_matrix* A, int64_t* info) {
  if (!A || !info) return GT_ERR_INVALID;
  info[0] = A->nbrows * A->bs;
  info[1] = A->bnnz * A->bs * A->bs;
  info[2] = A->bs;
  info[3] = A->precision;
  info[4] = A->nbrows;
  info[5] = A->bnnz;
  return GT_OK;
}

int gt_matrix_download_csr(gt_matrix* A, int64_t* rowptr, int32_t* colind, double* v64, float* v32) {
  if (!A) return GT_ERR_INVALID;
  Ctx* ctx = A->space->mesh->ctx;
  cudaSetDevice(ctx->device);
  int bs = A->bs;
  int64_t n = A->nbrows * bs, nnz = A->bnnz * bs * bs;
  int s = GT_OK;
  if (bs == 1) {
    if (rowptr) s = copy_out(ctx, rowptr, A->rowptr, n + 1);
    if (s == GT_OK && colind) s = copy_out(ctx, colind, A->colind, nnz);
    if (s == GT_OK && v64 && A->val64) s = copy_out(ctx, v64, A->val64, nnz);
    if (s == GT_OK && v32 && A->val32) s = copy_out(ctx, v32, A->val32, nnz);
  } else {
    int64_t* rp = nullptr;
    int32_t* ci = nullptr;
    double* d64 = nullptr;
    float* d32 = nullptr;
    if (rowptr) {
      s = dalloc(ctx, &rp, n + 1);
      if (s == GT_OK) {
        k_expand_rowptr<<<GT_KC(ctx, grid_for(n + 1, 256)), 256, 0, ctx->stream>>>(A->rowptr, A->nbrows, bs, rp);
        s = copy_out(ctx, rowptr, rp, n + 1);
      }
    }
    if (s == GT_OK && (colind || (v64 && A->val64))) {
      if (colind) s = dalloc(ctx, &ci, nnz);
      if (s == GT_OK && v64 && A->val64) s = dalloc(ctx, &d64, nnz);
      if (s == GT_OK) {
        k_expand_entries<double><<<GT_KC(ctx, (unsigned)A->nbrows), 128, 0, ctx->stream>>>(A->rowptr, A->colind, A->val64, A->nbrows,
                                                                             bs, ci, d64);
        if (colind) s = copy_out(ctx, colind, ci, nnz);
        if (s == GT_OK && d64) s = copy_out(ctx, v64, d64, nnz);
      }
    }
    if (s == GT_OK && v32 && A->val32) {
      s = dalloc(ctx, &d32, nnz);
      if (s == GT_OK) {
        k_expand_entries<float><<<GT_KC(ctx, (unsigned)A->nbrows), 128, 0, ctx->stream>>>(A->rowptr, A->colind, A->val32, A->nbrows,
                                                                            bs, nullptr, d32);
        s = copy_out(ctx, v32, d32, nnz);
      }
    }
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (s == GT_OK && e != cudaSuccess) s = check_cuda(ctx, e, "gt_matrix_download_csr");
    dfree(ctx, rp);
    dfree(ctx, ci);
    dfree(ctx, d64);
    dfree(ctx, d32);
    return s;
  }
  if (s == GT_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) s = check_cuda(ctx, e, "gt_matrix_download_csr");
  }
  return s;
}

int gt_matrix_destroy(gt_matrix* A) {
  if (!A) return GT_ERR_INVALID;
  matrix_release(A);
  delete A;
  return GT_OK;
}

}  // extern "C"
