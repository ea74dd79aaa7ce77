// gt_internal.cuh -- shared definitions of the GB300 assembly/solve library.
//
// Object model (all device state lives in HBM and is owned by a context):
//   gt_ctx    stream, buffer pool, error flag, last error message
//   gt_mesh   coords (node-major FP64), cell->nodes (0-based), parent faces
//   gt_space  node-level DOF ids per cell (1-based free, negative Dirichlet);
//             a vector space with ncomp components numbers DOF (node, comp)
//             as (node_dof-1)*ncomp + comp + 1, which is the reference's
//             component-major numbering when Dirichlet tags whole nodes
//   gt_matrix block CSR (block size = ncomp) sparsity plus FP64 and/or FP32
//             values; the incidence lists (block row -> (cell, local node))
//             drive the deterministic row-owner scatter
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/gtgpu.h"

namespace gt {

constexpr int kMaxNodesPerCell = 27;  // Q2 hexahedron
constexpr int kMaxLocal = 81;         // Q2 hexahedron, 3 components

struct Ctx;

// ---------------------------------------------------------------------------
// error plumbing
// ---------------------------------------------------------------------------
int set_error(Ctx* ctx, int code, const std::string& msg);
int check_cuda(Ctx* ctx, cudaError_t e, const char* what);
#define GT_CUDA(ctx, call)                                   \
  do {                                                       \
    cudaError_t e__ = (call);                                \
    if (e__ != cudaSuccess) return check_cuda(ctx, e__, #call); \
  } while (0)
#define GT_LAUNCH(ctx, what)                                         \
  do {                                                               \
    cudaError_t e__ = cudaGetLastError();                            \
    if (e__ != cudaSuccess) return check_cuda(ctx, e__, what);       \
  } while (0)
#define GT_TRY(expr)          \
  do {                        \
    int s__ = (expr);         \
    if (s__ != GT_OK) return s__; \
  } while (0)

// device-side error word bits (written with atomicOr, read by the host)
enum : uint32_t {
  DEV_ERR_NODE_RANGE = 1u,
  DEV_ERR_ROW_CAP = 2u,
  DEV_ERR_HASH_FULL = 4u,
  DEV_ERR_LOOKUP = 8u,
  DEV_ERR_DEGENERATE = 16u,
  DEV_ERR_KEY_RANGE = 32u,
};

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct Ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // copy stream: host<->device transfers that overlap the kernels of the
  // main stream (ordered against it with events)
  cudaStream_t side = nullptr;
  // second compute stream: element kernels that run beside the sparsity
  // kernels of the main stream (FP64-pipe work next to integer/shared-memory
  // work on the same SMs), joined with an event before the scatter
  cudaStream_t aux = nullptr;
  std::vector<cudaEvent_t> free_events;
  std::string err;
  // size-bucketed pool of device blocks (no cudaMalloc in steady state)
  std::multimap<size_t, void*> pool;
  std::unordered_map<void*, size_t> live;
  int64_t live_bytes = 0, pooled_bytes = 0;
  uint32_t* d_err = nullptr;       // device error word
  uint32_t* h_err = nullptr;       // pinned mirror
  uint32_t held_err = 0;           // bits taken by a pass that checks only its own, returned on the next take
  int64_t* h_scratch = nullptr;    // pinned small readbacks (64 words)
  double* h_dscratch = nullptr;    // pinned small FP64 readbacks (64 words)
  int64_t launches = 0;            // kernels launched by this context
  int64_t graph_launches = 0;      // CUDA-graph launches (replayed CG chunks)
  // PCG path: 0 = by size (persistent kernel for small systems, separate
  // launches per phase for large ones), 1 = always launches, 2 = always
  // persistent (environment GTGPU_PCG=launches|persistent at context creation)
  int pcg_path = 0;
  // element kernels on the auxiliary stream beside the sparsity kernels
  // (GTGPU_OVERLAP=0 at context creation: one stream, in order)
  bool overlap = true;
  // sparsity count pass with one thread per row where rows are short
  // (GTGPU_PATTERN=warps at context creation: one warp per row always)
  bool pattern_rows = true;
  // affine QUAD4/HEX8 meshes whose cells all share one geometry record (to
  // 1e-13 relative) scatter scale_c x one reference element block
  // (GTGPU_UNIFORM=0 at context creation: always the per-cell records)
  bool uniform_geom = true;
  // mixed-precision hand-over: an FP32 cycle (between two reliable updates)
  // whose FP64 true residual norm^2 did not fall below ir_stall_ratio x its
  // value at the cycle start counts as stalled; ir_stall_count stalled cycles
  // in a row continue the solve in FP64 (GTGPU_IR_STALL="ratio,count" at
  // context creation)
  double ir_stall_ratio = 0.25;
  int ir_stall_count = 3;
  // reliable update when the FP32 recurrence residual norm fell by this
  // factor since the last one (GTGPU_IR_DELTA at context creation).  0.3
  // measured: Q2 elasticity 64^3 5244 FP32 iterations (0.1: 7049), the P1
  // Poisson 96^3 x 6 solve 2% slower (20 updates instead of 11)
  double ir_delta = 0.3;
  // FP64-valued P1 element matrices computed in double-float on the FP32
  // pipes (GTGPU_P1=fp64 at context creation: the FP64-pipe kernel)
  bool p1_dfloat = true;
  // lanes per row of the CSR row kernels: 0 = from the mean row length,
  // else 1, 2, 4 or 8 (GTGPU_SPMV_LANES at context creation)
  int spmv_lanes = 0;
  // phase profiling: CUDA events recorded on the stream between phases
  bool prof = false;
  std::vector<std::pair<std::string, cudaEvent_t>> marks;
  std::vector<cudaEvent_t> spare_events;
};

// events without timing, recycled by the context
cudaEvent_t event_get(Ctx* ctx);
void event_put(Ctx* ctx, cudaEvent_t e);
// Copies bytes from a host pointer to device memory on the copy stream,
// after the work already queued on the main stream (so a buffer still read
// by queued kernels is not overwritten early).  *done receives the event the
// main stream must wait on before using dst.  A pinned source may still be
// read after the call returns.
int side_copy_in(Ctx* ctx, void* dst, const void* src, size_t bytes, cudaEvent_t* done);

// counts a kernel launch; used as the grid argument: k<<<GT_KC(ctx, g), ...>>>
#define GT_KC(ctx, g) ((ctx)->launches++, (g))

// records a named phase boundary when profiling is on
void mark(Ctx* ctx, const char* name);

void* pool_alloc(Ctx* ctx, size_t bytes);
void pool_free(Ctx* ctx, void* p);
void pool_trim(Ctx* ctx);

template <class T>
int dalloc(Ctx* ctx, T** out, int64_t n) {
  size_t bytes = (size_t)(n > 0 ? n : 1) * sizeof(T);
  void* p = pool_alloc(ctx, bytes);
  if (!p) {
    *out = nullptr;
    return set_error(ctx, GT_ERR_OOM, "device allocation of " + std::to_string(bytes) + " bytes failed");
  }
  *out = (T*)p;
  return GT_OK;
}
template <class T>
void dfree(Ctx* ctx, T*& p) {
  if (p) pool_free(ctx, (void*)p);
  p = nullptr;
}

// reads the device error word (synchronises the stream) and clears it
int take_device_error(Ctx* ctx, uint32_t* bits);

// copy n elements from a host or device pointer (unified addressing)
template <class T>
int copy_in(Ctx* ctx, T* dst, const T* src, int64_t n) {
  if (n <= 0) return GT_OK;
  GT_CUDA(ctx, cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyDefault, ctx->stream));
  return GT_OK;
}
template <class T>
int copy_out(Ctx* ctx, T* dst, const T* src, int64_t n) {
  if (n <= 0) return GT_OK;
  GT_CUDA(ctx, cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyDefault, ctx->stream));
  return GT_OK;
}

// ---------------------------------------------------------------------------
// mesh / space / matrix
// ---------------------------------------------------------------------------
struct Mesh {
  Ctx* ctx = nullptr;
  int ctype = 0, D = 0, nv = 0;  // cell type, dimension, nodes per cell
  int64_t nnodes = 0, ncells = 0;
  double* coords = nullptr;      // nnodes * D
  int32_t* cell_nodes = nullptr; // ncells * nv, 0-based
  int64_t ncorners = 0;
  int32_t* corners = nullptr;    // 0-based
  int64_t nbfaces = 0;
  int nbfv = 0;                  // nodes per boundary face
  int32_t* bfaces = nullptr;     // 0-based
  int32_t* bgroup = nullptr;
  int64_t nbedges = 0;
  int32_t* bedges = nullptr;     // 3-D parent 1-faces, 0-based
  // coordinates uploaded on the copy stream: kernels reading coords wait
  cudaEvent_t coords_ev = nullptr;
  bool coords_pending = false;
};

// orders the main stream after a pending coordinate upload of the mesh
void mesh_wait_coords(Mesh* m);
// orders stream s after it too (the upload stays pending for the main stream)
void mesh_wait_coords_on(Mesh* m, cudaStream_t s);

struct Space {
  Ctx* ctx = nullptr;  // owning context (also reachable as mesh->ctx while the mesh lives)
  Mesh* mesh = nullptr;
  int order = 1, ncomp = 1, nn = 0, nloc = 0;
  int64_t nfree_nodes = 0, ndiri_nodes = 0;
  int32_t* cell_ndofs = nullptr;  // ncells * nn: node-level dof, >0 free (1-based), <0 Dirichlet
  // largest difference of two free node DOFs of one cell (-1: not known): a
  // bound on |column - row| in every row of the space's matrices
  int32_t dof_spread = -1;
  // incidence cache used by stand-alone vector assembly
  int64_t* inc_ptr = nullptr;
  int32_t* inc = nullptr;
  int64_t ninc = 0;
};

// row chunks of the pipelined scatter (and of its downloads to host buffers)
constexpr int kRowChunks = 8;

struct Matrix {
  Ctx* ctx = nullptr;  // owning context
  Space* space = nullptr;
  int bs = 1, precision = GT_FP64;
  int64_t nbrows = 0, bnnz = 0;
  int max_row = 0;                 // longest block row
  int64_t* rowptr = nullptr;       // nbrows + 1
  int32_t* colind = nullptr;       // bnnz, 0-based block columns
  double* val64 = nullptr;         // bnnz * bs * bs (row-major blocks)
  float* val32 = nullptr;
  int64_t* inc_ptr = nullptr;      // block row -> incidences
  int32_t* inc = nullptr;          // cell * nn + local node
  int64_t ninc = 0;
  int32_t* diag_pos = nullptr;     // position of the diagonal block in each row
  // sliced-ELL copy of a scalar matrix for the SpMV (32-row slices, see
  // gt_solve.cu): built on first use, values refreshed after every update
  int sell_state = 0;              // 0 not built, 1 built, -1 not taken (padding)
  int64_t sell_nslices = 0, sell_total = 0;
  int64_t* sell_ptr = nullptr;     // nslices + 1
  int32_t* sell_len = nullptr;     // nslices
  int32_t* sell_col = nullptr;
  double* sell_v64 = nullptr;
  float* sell_v32 = nullptr;
  bool sell_cur64 = false, sell_cur32 = false;  // values match val64 / val32
  // the last cell among the incidences of each row chunk (rows nbrows*k/K ..
  // nbrows*(k+1)/K, K = kRowChunks; -1: no incidence), from the count pass:
  // the scatter of a chunk waits only for the element chunks up to that cell
  int32_t chunk_last[kRowChunks] = {};
  bool chunk_last_ok = false;
};

// called by every kernel launch that rewrites a matrix's values
inline void matrix_values_changed(Matrix* A) {
  A->sell_cur64 = false;
  A->sell_cur32 = false;
}
// frees the sliced-ELL copy
void sell_release(Matrix* A);

// ---------------------------------------------------------------------------
// library-internal entry points (implemented across the .cu files)
// ---------------------------------------------------------------------------
int number_dofs(Space* sp, int ngroups, const int32_t* groups);
// incidence lists; sort = false leaves the order to the sparsity count pass
int build_incidence(Ctx* ctx, const Space* sp, int64_t** inc_ptr, int32_t** inc, int64_t* ninc, bool sort);
// the same for any array of n node-level DOF ids (>0 free) over nrows rows
int build_incidence_arr(Ctx* ctx, const int32_t* dofs, int64_t n, int64_t nrows, int64_t** inc_ptr, int32_t** inc,
                        int64_t* ninc, bool sort);
// the matrix's incidence (A->inc_ptr, A->inc: every row's list ascending) and
// its sparsity (rowptr, colind, max_row); chunk_last: also each row chunk's
// last cell (Matrix::chunk_last)
int build_pattern(Matrix* A, bool chunk_last = false);
// Element matrices of scalar P1 tetrahedra (Laplacian, mass) are symmetric
// and stored packed: the 10 entries of the upper triangle per cell, row by
// row ({00,01,02,03,11,12,13,22,23,33}); every other space stores the full
// nloc x nloc row-major block per cell.
inline bool ke_packed(const Space* sp) {
  return sp->mesh->ctype == GT_TET4 && sp->order == 1 && sp->ncomp == 1;
}
// entries of the element-matrix buffer per cell
inline int64_t ke_per_cell(const Space* sp) { return ke_packed(sp) ? 10 : (int64_t)sp->nloc * sp->nloc; }
// keep_tab (optional): receives the tabulation buffer the kernels read
// instead of freeing it (for launches on a stream other than the main one,
// whose reuse of the block must wait for them)
// Element kernels launched over cell chunks, each followed by its event (so
// a consumer can start on the first chunks): n events in, n chunks out; a
// path without chunked launches sets n = 0.
struct ElemChunks {
  int n = 0;
  int64_t end[kRowChunks] = {};  // chunk i covers cells [end[i-1], end[i])
  cudaEvent_t ev[kRowChunks] = {};
};
int compute_elements(const Space* sp, int form, const double* d_coef, double nu, int precision,
                     const double* f, const double* d_scoef, void* Ke, double* be, int want_matrix,
                     double** keep_tab = nullptr, ElemChunks* chunks = nullptr);
// be/bvec (optional): element vectors and the load vector summed in the same
// pass; xd: Dirichlet values (lift); [r0, r1): block rows (r1 < 0: all)
int scatter_matrix(Matrix* A, const void* Ke, int ke_precision, int out_precision, const double* be = nullptr,
                   double* bvec = nullptr, const double* xd = nullptr, int64_t r0 = 0, int64_t r1 = -1);
int tabulation_doubles(const Space* sp);
int compute_elements_with_tab(const Space* sp, int form, const double* d_coef, double nu, int precision,
                              double* tab, void* Ke);
int scatter_vector(const Space* sp, const int64_t* inc_ptr, const int32_t* inc, const double* be,
                   double* b);
int find_diag(Matrix* A);
int solve(Matrix* A, const double* b, double* x, double rtol, int maxit, int mode, gt_solve_info* info);
// Mixed-precision CG: a reliable-update cycle (recurrence residual down by
// a decade) of more than kSlowCycle FP32 iterations means cond(A) >~ 1e6 in
// CG terms (about 1.15 sqrt(cond) iterations per decade), where eps32 *
// cond(A) ~ 0.1 slows the FP32 iteration several-fold below the FP64 rate;
// the solve then continues in FP64.  Also a cycle 2.5x longer than the
// longest earlier one, or three updates that did not halve the true
// residual.  (Measured: problems at 300-450 FP32 iterations per decade still
// gain from FP32; one at ~2500 per decade needed 4x the FP64 count.)
constexpr int kSlowCycle = 1000;
// A true-residual check whose r.z exceeds the recurrence's by this factor
// restarts the CG directions from the true residual (beta = 0): the
// recurrence has drifted.  kRestartRatio64 for the FP64 iteration, whose
// checks come only when the recurrence claims convergence (a mismatch there
// means the recurrence ran past the attainable accuracy, and scaling the
// old direction by it corrupts the iteration), kRestartRatio for the
// periodic reliable updates of the FP32 iteration.
constexpr double kRestartRatio = 100.0;
constexpr double kRestartRatio64 = 4.0;
// FP64 CG ends (not converged) after this many true-residual checks in a row
// that did not halve the residual norm: the tolerance is below what
// eps64 * cond(A) allows.
constexpr int kStagnation = 3;

// persistent cooperative Jacobi-PCG (gt_pcg.cu); x holds the start value
int pcg_persistent(Matrix* A, int mode, const double* b, double* x, double rtol, int maxit, int32_t* iters,
                   int32_t* nupd, int32_t* iters64, double* relres);
// scalar rows up to which a system is solved by the persistent kernel
constexpr int64_t kPersistentMaxRows = 262144;
// pcg_persistent for several systems of ctx at once (GT_SOLVE_FP64 or
// GT_SOLVE_IR), in shared cooperative launches; results bitwise those of
// pcg_persistent on each system alone
int pcg_persistent_groups(Ctx* ctx, const std::vector<Matrix*>& As, int mode, const std::vector<const double*>& b,
                          const std::vector<double*>& x, double rtol, int maxit, std::vector<gt_solve_info>& infos,
                          std::vector<int>& status);
int spmv64(Matrix* A, const double* x, double* y);
// the persistent solver's grid barrier run alone (gt_pcg.cu): ctas CTAs wait
// for ctas + missing arrivals with the given time limit
int barrier_probe(Ctx* ctx, int ctas, int missing, int64_t timeout_ns);

// device scans (exclusive prefix sum; out has n+1 entries, out[n] = total)
int exclusive_scan_i64(Ctx* ctx, const int32_t* in, int64_t* out, int64_t n);
int exclusive_scan_i32(Ctx* ctx, const int32_t* in, int32_t* out, int64_t n);

inline int grid_for(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > 2147483647LL) g = 2147483647LL;
  return (int)g;
}

inline int space_nodes(int ctype, int order) {
  if (ctype == GT_TET4) return order == 2 ? 10 : 4;
  int D = ctype == GT_QUAD4 ? 2 : 3;
  int m = order + 1;
  return D == 2 ? m * m : m * m * m;
}

}  // namespace gt

// opaque ABI handles are the internal structs
struct gt_ctx : gt::Ctx {};
struct gt_mesh : gt::Mesh {};
struct gt_space : gt::Space {};
struct gt_matrix : gt::Matrix {};
