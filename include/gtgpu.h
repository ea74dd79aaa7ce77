/*
 * gtgpu.h -- C ABI of the GB300 finite-element assembly + solve library.
 *
 * The entry points replace the problem-level seam of GalerkinToolkit.jl
 * (v0.6.3).  Each declaration names the reference interface it stands in
 * for (paths are inside the GalerkinToolkit.jl source tree).
 *
 * Conventions
 *  - Every function returns an int status: GT_OK (0) or a negative GT_ERR_*.
 *    Nothing aborts; gt_last_error(ctx) gives the message of the last error.
 *  - Pointer arguments may be host (pageable or pinned) or device pointers;
 *    the library copies through unified addressing.  Output pointers that
 *    refer to host memory are complete when the call returns.
 *  - Ids follow GalerkinToolkit (src/helpers.jl:47-61): node ids in
 *    cell_nodes and boundary-face arrays are 1-based Int32; DOF ids returned
 *    by gt_space_cell_dofs are 1-based for free DOFs and negative for
 *    Dirichlet DOFs (src/space.jl:515-524).  CSR arrays are 0-based
 *    (rowptr int64, colind int32); a Julia caller adds 1 when it wraps them
 *    as SparseMatrixCSC (the matrix is symmetric, so CSR == CSC).
 *  - One context per host thread (or serialise calls).  All work of a
 *    context runs on its CUDA stream, in call order.
 */
#ifndef GTGPU_H
#define GTGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GT_OK 0
#define GT_ERR_INVALID (-1)       /* bad argument or malformed mesh */
#define GT_ERR_CUDA (-2)          /* CUDA runtime error */
#define GT_ERR_OOM (-3)           /* device allocation failed */
#define GT_ERR_UNSUPPORTED (-4)   /* weak form / element outside the supported set */
#define GT_ERR_NOT_CONVERGED (-5) /* iterative solve hit maxit */
#define GT_ERR_TIMEOUT (-6)       /* a bounded device-side wait gave up */
#define GT_ERR_BUDGET (-7)        /* request refused by the HBM admission budget */

/* cell types (geometry) */
#define GT_QUAD4 1
#define GT_HEX8 2
#define GT_TET4 3

/* weak forms (the only ones supported; anything else is GT_ERR_UNSUPPORTED) */
#define GT_LAPLACE 1    /* int coef * grad(u) . grad(v) */
#define GT_MASS 2       /* int coef * u v */
#define GT_ELASTICITY 3 /* int sigma(eps(u)) : eps(v), E = coef, Poisson ratio nu */

/* precision of the assembled values */
#define GT_FP64 0  /* FP64 integration, FP64 values */
#define GT_FP32 1  /* FP64 Jacobian inverse/determinant, FP32 element matrix and values */
#define GT_MIXED 2 /* FP64-integrated FP64 values (the outer residual) plus FP32-integrated
                      FP32 values (the inner CG), sharing the index arrays */

/* solve modes */
/* Convergence of GT_SOLVE_FP64 and GT_SOLVE_IR is decided on the FP64 true
 * residual ||b - A x|| <= rtol ||b||. */
#define GT_SOLVE_FP64 0 /* Jacobi-PCG in FP64 */
#define GT_SOLVE_IR 1   /* Jacobi-PCG in FP32 with FP64 reliable updates: the
                           FP64 true residual and solution replace the FP32
                           recurrence whenever its residual fell tenfold */
#define GT_SOLVE_FP32 2 /* Jacobi-PCG in FP32 (needs FP32 values) */

typedef struct gt_ctx gt_ctx;
typedef struct gt_mesh gt_mesh;
typedef struct gt_space gt_space;
typedef struct gt_matrix gt_matrix;

typedef struct gt_solve_info {
  int32_t iterations;       /* PCG iterations */
  int32_t outer_iterations; /* FP64 true-residual updates (GT_SOLVE_FP64/IR), else 0 */
  double rel_residual;      /* final ||b - A x|| / ||b|| in FP64 */
  int32_t fp64_iterations;  /* iterations run in FP64 (all of GT_SOLVE_FP64; in GT_SOLVE_IR
                               those after an FP32 stall, when eps32 * cond(A) ~ 1) */
  int32_t reserved;
} gt_solve_info;

/* ---- context ------------------------------------------------------------ */
/* No reference counterpart (the reference is a single-process CPU library);
 * owns the CUDA stream, the buffer pool and the last error message. */
int gt_ctx_create(int device, gt_ctx** ctx);
int gt_ctx_destroy(gt_ctx* ctx);
const char* gt_last_error(const gt_ctx* ctx);
int gt_ctx_synchronize(gt_ctx* ctx);
/* Use an external stream (cudaStream_t passed as void*); NULL restores the
 * context's own stream (created at the highest priority).  The context runs
 * element kernels on a second, lowest-priority stream beside the sparsity
 * kernels only when the main stream has a higher priority than that one;
 * with a default-priority external stream the phases run in order. */
int gt_ctx_set_stream(gt_ctx* ctx, void* stream);
/* Bytes of device memory currently held by the context (live + pooled). */
int gt_ctx_memory(gt_ctx* ctx, int64_t* live_bytes, int64_t* pooled_bytes);
/* Returns the pooled (free) device blocks of the context to the driver. */
int gt_ctx_trim(gt_ctx* ctx);
/* Measured FMA throughput of the device in TFLOP/s (GT_FP64 or GT_FP32);
 * the roofline of the integration kernels.  No reference counterpart. */
int gt_ctx_fma_rate(gt_ctx* ctx, int precision, double* tflops);
/* Failure-detection check of the persistent solver's grid barrier, no
 * reference counterpart: `ctas` co-resident CTAs run the barrier the
 * persistent PCG uses between its phases, waiting for ctas + missing
 * arrivals with a time limit of timeout_ns (at most 2 s).  missing = 0
 * completes (GT_OK); missing > 0 can never complete, so every CTA gives up
 * after the limit and the call returns GT_ERR_TIMEOUT with the context still
 * usable -- the path a solve takes when a barrier does not complete. */
int gt_ctx_barrier_probe(gt_ctx* ctx, int ctas, int missing, int64_t timeout_ns);
/* Number of kernels the context has launched so far. */
int gt_ctx_launch_count(gt_ctx* ctx, int64_t* launches);
/* Number of CUDA-graph launches the context has made so far (the solver
 * replays each chunk of CG iterations as one captured graph). */
int gt_ctx_graph_launch_count(gt_ctx* ctx, int64_t* launches);
/* Phase timing with CUDA events on the context's stream: begin, run calls,
 * end.  end() returns up to max phases: names (32 chars each) and device
 * milliseconds between consecutive phase boundaries. */
int gt_ctx_profile_begin(gt_ctx* ctx);
int gt_ctx_profile_end(gt_ctx* ctx, int max, char* names, double* ms, int* count);

/* ---- mesh --------------------------------------------------------------- */
/* Replaces GT.mesh(...) of a cartesian_mesh (src/mesh.jl:573-650,
 * src/cartesian_mesh.jl:16-54): node coordinates (node-major, nnodes*D),
 * cell->nodes (1-based, local node order of the reference cell), the parent
 * 0-faces (corner nodes), the parent (D-1)-faces with their group index k
 * (group "(D-1)-face-k"), and in 3-D the parent 1-faces (box-edge
 * segments).  Parent faces fix the topology numbering of complexify
 * (src/topology.jl:1034-1125). */
int gt_mesh_create(gt_ctx* ctx, int cell_type, int64_t nnodes, const double* coords,
                   int64_t ncells, const int32_t* cell_nodes, int64_t ncorners,
                   const int32_t* corner_nodes, int64_t nbfaces, const int32_t* bface_nodes,
                   const int32_t* bface_group, int64_t nbedges, const int32_t* bedge_nodes,
                   gt_mesh** mesh);
/* Replaces GT.replace_node_coordinates (src/mesh.jl:698-713) in place.  A
 * host source is uploaded on the context's copy stream, ordered before every
 * later use of the coordinates; a pinned source must stay unchanged until
 * the next call that returns results to the host. */
int gt_mesh_set_coords(gt_mesh* mesh, const double* coords);
int gt_mesh_destroy(gt_mesh* mesh);

/* ---- space / DOF numbering ---------------------------------------------- */
/* Replaces GT.lagrange_space(Omega, order; tensor_size, dirichlet_boundary)
 * (src/space.jl:1702-1735) and its generate_dof_ids (src/space.jl:299-535),
 * computed on the device.  order 1 or 2 (Q1/Q2 on QUAD4/HEX8, P1/P2 on TET4), ncomp 1 or D.
 * ngroups: -1 = Dirichlet on all boundary faces (GT.boundary(mesh)),
 * 0 = no Dirichlet, >0 = the groups listed in `groups` (values k of
 * "(D-1)-face-k").  Vector spaces are clamped on all components. */
int gt_space_create(gt_mesh* mesh, int order, int ncomp, int ngroups, const int32_t* groups,
                    gt_space** space);
/* info[0]=num_free_dofs info[1]=num_dirichlet_dofs info[2]=local dofs per
 * cell info[3]=ncells info[4]=free nodes (block rows) info[5]=ncomp */
int gt_space_info(const gt_space* space, int64_t* info);
/* GT.face_dofs(V) (src/space.jl:1820-1853): ncells*nloc, GT convention. */
int gt_space_cell_dofs(const gt_space* space, int32_t* cell_dofs);
int gt_space_destroy(gt_space* space);

/* ---- matrix assembly ---------------------------------------------------- */
/* Replaces GT.assemble_matrix(a, T, V, V; reuse=Val(true))
 * (src/problems.jl:319-350): sparsity (allocate_matrix counting pass and
 * COO->CSC compress, src/assembly.jl:75-153,571-575) plus values of the
 * form, in one call.  cell_coef: per-cell coefficient (ncells) or NULL
 * (= 1); nu: Poisson ratio (GT_ELASTICITY only).  The returned matrix keeps
 * the sparsity so gt_update_matrix can refill values. */
int gt_assemble_matrix(gt_space* space, int form, const double* cell_coef, double nu, int precision,
                       gt_matrix** matrix);
/* Replaces GT.assemble_matrix_and_vector(a, l, T, U, V; reuse=Val(true))
 * (src/problems.jl:391-407): the matrix as gt_assemble_matrix plus the
 * vector of int source_coef*f.v (f: ncomp values; source_coef per cell or
 * NULL = 1) into b (num_free_dofs FP64), sharing one sparsity construction. */
int gt_assemble_matrix_and_vector(gt_space* space, int form, const double* cell_coef, double nu,
                                  int precision, const double* f, const double* source_coef, double* b,
                                  gt_matrix** matrix);
/* Replaces GT.PartitionedSolvers_linear_problem(uhd, a, l) with Dirichlet
 * data (src/problems.jl:439-453): assembles A (free x free) and the load
 * vector, and subtracts the Dirichlet lift Ad * xd (Ad = free x Dirichlet
 * columns of the form) in the same pass, without assembling Ad.
 * dirichlet_values: num_dirichlet_dofs values in the Dirichlet numbering
 * (DOF -k -> dirichlet_values[k-1]), e.g. the interpolated boundary data;
 * b receives b - Ad * xd.  f and b are required. */
int gt_linear_problem(gt_space* space, int form, const double* cell_coef, double nu, int precision,
                      const double* f, const double* source_coef, const double* dirichlet_values, double* b,
                      gt_matrix** matrix);
/* GT.assemble_matrix_and_vector returning the host CSR arrays in one call
 * (the reference returns a host SparseMatrixCSC, src/problems.jl:391-414):
 * assembles like gt_assemble_matrix_and_vector and fills rowptr (rows + 1,
 * int64), colind and values64 / values32 (either may be NULL) with the
 * scalar CSR.  capacity: entries colind / values can hold; a smaller
 * capacity returns GT_ERR_INVALID (gt_matrix_info gives the count of a
 * previous assembly of the same space).  Host inputs are uploaded, and the
 * pattern downloaded, on a copy stream while the device works on other
 * phases: with pinned host buffers the transfers overlap the kernels. */
int gt_assemble_csr(gt_space* space, int form, const double* cell_coef, double nu, int precision, const double* f,
                    const double* source_coef, double* b, int64_t capacity, int64_t* rowptr, int32_t* colind,
                    double* values64, float* values32, gt_matrix** matrix);
/* Replaces GT.update_matrix!(A, cache) (src/problems.jl:352-361): new values
 * on the existing sparsity. */
int gt_update_matrix(gt_matrix* matrix, int form, const double* cell_coef, double nu);
/* No counterpart in the reference.  gt_update_matrix without allocating:
 * for callers that must not have the library allocate device memory (a
 * process whose device memory is budgeted up front by its own admission
 * control or memory pool, or a latency-critical refill loop where
 * cudaMalloc/cudaFree can synchronise the device).  Refills the values of an
 * assembled matrix using one static 128 MiB device array as scratch (a
 * GT_MIXED matrix gets its FP32 values as the rounded FP64 values, in the
 * same pass); cell_coef must be device memory of the matrix's device or
 * NULL; a refill needing more scratch
 * than 128 MiB (tabulation + ncells*nloc^2 values) returns GT_ERR_INVALID.
 * The first call on a device looks up the array's address; every call
 * waits for the context's stream before it returns.  All calls on a device share the one array, which keeps the last
 * call's contents: calls that overlap on the GPU (two streams, contexts or
 * threads at once) race on it, so callers serialise them. */
int gt_update_matrix_noalloc(gt_matrix* matrix, int form, const double* cell_coef, double nu);
/* Replaces GT.update_matrix_and_vector! (src/problems.jl:409-414). */
int gt_update_matrix_and_vector(gt_matrix* matrix, int form, const double* cell_coef, double nu,
                                const double* f, const double* source_coef, double* b);
/* info[0]=rows info[1]=nnz (scalar) info[2]=block size info[3]=precision
 * info[4]=block rows info[5]=block nnz */
int gt_matrix_info(const gt_matrix* matrix, int64_t* info);
/* Scalar CSR of the free x free matrix.  Any output may be NULL; the
 * values arrays are filled only if the matrix holds that precision. */
int gt_matrix_download_csr(gt_matrix* matrix, int64_t* rowptr, int32_t* colind, double* values_f64,
                           float* values_f32);
int gt_matrix_destroy(gt_matrix* matrix);

/* ---- integrals ----------------------------------------------------------- */
/* Replaces GT.assemble_scalar (src/problems.jl:172-190) for the integrands
 * the reference's tests integrate: the sum over the cells of
 *   GT_INT_VOLUME    int 1
 *   GT_INT_POLY      int p(x)
 *   GT_INT_FIELD     int sum_k u_k
 *   GT_INT_L2_NORM2  int sum_k u_k^2
 *   GT_INT_L2_ERROR2 int sum_k (u_k - p_k(x))^2
 *   GT_INT_H1_ERROR2 int sum_k |grad u_k - grad p_k(x)|^2
 * with the space's quadrature (degree 2 * order).  u: the discrete field,
 * u_free (num_free_dofs values) and u_dirichlet (the Dirichlet DOF values,
 * DOF -k -> u_dirichlet[k-1]; NULL = 0); p_k: a quadratic with 10
 * coefficients (of 1, x, y, z, x^2, y^2, z^2, xy, xz, yz) per component
 * (one set for GT_INT_POLY).  Host or device inputs; result on the host;
 * the cell sums are added in a fixed order (bitwise reproducible). */
#define GT_INT_VOLUME 0
#define GT_INT_POLY 1
#define GT_INT_FIELD 2
#define GT_INT_L2_NORM2 3
#define GT_INT_L2_ERROR2 4
#define GT_INT_H1_ERROR2 5
int gt_integrate(gt_space* space, int kind, const double* u_free, const double* u_dirichlet, const double* poly,
                 double* result);

/* ---- vector assembly ---------------------------------------------------- */
/* Replaces GT.assemble_vector(v -> int f*v dOmega, T, V) (src/problems.jl:
 * 244-274, src/assembly.jl:27-73,558-569) with a constant source f (ncomp
 * values) times an optional per-cell coefficient.  b: num_free_dofs FP64. */
int gt_assemble_vector(gt_space* space, const double* f, const double* cell_coef, double* b);
/* Replaces GT.assemble_vector(v -> int g v dGamma, T, V) over boundary faces
 * (the Neumann term of docs/src/src_jl/example_poisson_equation.jl:161-203;
 * src/problems.jl:244-274 with a boundary measure): a constant g (ncomp
 * values) on the boundary faces of the groups (k of "(D-1)-face-k"; ngroups
 * < 0: every boundary face).  b: num_free_dofs FP64 (host or device);
 * accumulate != 0 adds to b.  Each DOF sums its faces in (cell, local face)
 * order. */
int gt_assemble_boundary_vector(gt_space* space, int ngroups, const int32_t* groups, const double* g, double* b,
                                int accumulate);

/* ---- solve -------------------------------------------------------------- */
/* Replaces PS.solve(PS.LinearAlgebra_lu(GT.PartitionedSolvers_linear_problem
 * (...))) (src/problems.jl:439-462) with a Jacobi-preconditioned CG (the
 * reference has no CG of its own).  b, x: num_free_dofs FP64; x holds the
 * initial guess on entry.  rtol on ||b - A x|| / ||b||. */
int gt_solve(gt_matrix* matrix, const double* b, double* x, double rtol, int maxit, int mode,
             gt_solve_info* info);
/* y = A x in the matrix's FP64 values (or FP32 when it has no FP64). */
int gt_spmv(gt_matrix* matrix, const double* x, double* y);

/* ---- batched solves ----------------------------------------------------- */
/* No counterpart in the reference (which solves one problem per call).
 * A batch of n assembled matrices of block size 1 (scalar problems) or 3
 * (3-D elasticity) on the device of ctx (they may come from other contexts
 * of that device, e.g. assembled concurrently on several streams), solved
 * together on ctx's stream: instances of up to 32768 scalar rows (see
 * gt_batch_set_small_rows) in one persistent launch per block size in which
 * each CTA takes instances from a queue (largest first) and runs each one's
 * whole Jacobi-PCG alone; medium ones in grouped persistent launches (below);
 * larger ones one after the other through the single-system solver.  An
 * instance's result does not depend on the rest of the batch.  b and x are
 * the instances' vectors concatenated in batch order (num_free_dofs each,
 * FP64); x is the output (every solve starts from 0).  infos: n entries.
 * GT_SOLVE_IR needs GT_MIXED matrices.  Other block sizes: GT_ERR_INVALID. */
typedef struct gt_batch gt_batch;
int gt_batch_create(gt_ctx* ctx, int n, gt_matrix* const* matrices, gt_batch** batch);
/* lanes per matrix row in the SpMV of the one-CTA-per-instance solves (1, 2,
 * 4 or 8; 0, the default: each instance's own, from its mean row length;
 * block rows of 3 take 2 or 4: 1 -> 2, 8 -> 4) */
int gt_batch_set_lanes(gt_batch* batch, int lanes);
/* scalar rows up to which an instance is solved by one CTA (0 .. 32768; the
 * default 32768); larger ones up to 262,144 rows, of ctx's own matrices,
 * share grouped persistent launches in GT_SOLVE_FP64 / GT_SOLVE_IR mode,
 * each bitwise as its own gt_solve would give */
int gt_batch_set_small_rows(gt_batch* batch, int64_t rows);
/* info[0]=instances info[1]=total scalar rows info[2]=instances solved one per CTA
 * info[3]=lanes */
int gt_batch_info(const gt_batch* batch, int64_t* info);
int gt_batch_solve(gt_batch* batch, const double* b, double* x, double rtol, int maxit, int mode,
                   gt_solve_info* infos);
int gt_batch_destroy(gt_batch* batch);

/* ---- device buffers and served-request inputs --------------------------- */
/* No counterpart in the reference.  Device memory from ctx's buffer pool
 * (bytes >= 0; freed back to the pool, ordered after the work already
 * queued on ctx); a synchronous copy in any direction on ctx's stream. */
int gt_device_alloc(gt_ctx* ctx, int64_t bytes, void** out);
int gt_device_free(gt_ctx* ctx, void* ptr);
int gt_device_copy(gt_ctx* ctx, void* dst, const void* src, int64_t bytes);
/* The seeded per-cell coefficient of a served request, generated on the
 * device on ctx's stream: out[c] = exp(sigma z_c), z_c =
 * sqrt(-2 log(1 - u(2c))) cos(2 pi u(2c + 1)), u(k) = (splitmix64(s ^ k)
 * >> 11) 2^-53 with s = seed ^ 0xC0EFF1C1E47 -- the host generator of the
 * Python package (gtgpu.lognormal_cells) up to the last bits of log, cos and
 * exp.  out: device memory of ctx's device, ncells doubles. */
int gt_lognormal_cells(gt_ctx* ctx, int64_t ncells, double sigma, uint64_t seed, double* out);

#ifdef __cplusplus
}
#endif
#endif /* GTGPU_H */
