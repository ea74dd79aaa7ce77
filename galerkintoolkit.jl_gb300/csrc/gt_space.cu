// gt_space.cu -- mesh upload and device DOF numbering.
//
// Restates on the device what GalerkinToolkit computes sequentially:
//  * vertex ids (create_vertices!, src/topology.jl:1034-1097): nodes of the
//    parent 0-faces first in parent order, then every other node in node
//    order -- a flag + exclusive scan;
//  * edge and face ids for Q2 (generate_face_boundary, src/topology.jl:
//    1594-1704): parent faces keep ids 1..npar, every other face gets the
//    next id in the order in which the scan over the higher-dimensional
//    faces first meets it.  On the device: a hash table keyed by the face's
//    sorted vertices collects, per face, the minimum scan rank of its
//    instances (atomicMin); a flag at that rank + exclusive scan gives the
//    new ids in first-encounter order -- the sequential order, recovered
//    without a sequential scan;
//  * DOF offsets per d-face (generate_dof_ids_step_1, src/space.jl:327-466)
//    and the free-first / negative-Dirichlet renumbering of step_2
//    (src/space.jl:477-535, partition_from_mask :910-920) -- flags + scans.
#include <climits>
#include <cstring>

#include "gt_internal.cuh"
#include "gt_refcell.cuh"

namespace gt {

constexpr unsigned long long EMPTY_KEY = ~0ull;

__device__ __forceinline__ void sort3(int32_t& a, int32_t& b, int32_t& c) {
  int32_t t;
  if (a > b) { t = a; a = b; b = t; }
  if (b > c) { t = b; b = c; c = t; }
  if (a > b) { t = a; a = b; b = t; }
}

// Key of a face given its vertex ids: 2 vertices -> (min, max) in 32-bit
// halves; 3 or 4 vertices -> the 3 smallest ids in 21-bit fields (three
// vertices determine a triangle or a quadrilateral of a conforming mesh).
__device__ __forceinline__ unsigned long long face_key(const int32_t* v, int n, uint32_t* err) {
  if (n == 2) {
    int32_t a = v[0] < v[1] ? v[0] : v[1], b = v[0] < v[1] ? v[1] : v[0];
    return ((unsigned long long)(uint32_t)a << 32) | (uint32_t)b;
  }
  int32_t a = v[0], b = v[1], c = v[2];
  sort3(a, b, c);
  if (n == 4) {
    int32_t d = v[3];
    if (d < c) { c = d; sort3(a, b, c); }
  }
  if (c >= (1 << 21)) { atomicOr(err, DEV_ERR_KEY_RANGE); return EMPTY_KEY - 1; }
  return ((unsigned long long)a << 42) | ((unsigned long long)b << 21) | (unsigned long long)c;
}

struct Hash {
  unsigned long long* keys;
  int32_t* vals;
  int32_t* rank;
  int64_t cap;  // power of two
};

__device__ __forceinline__ uint64_t mix64(unsigned long long x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
  return x;
}

__device__ int64_t hash_insert(Hash h, unsigned long long key, uint32_t* err) {
  uint64_t s = mix64(key) & (uint64_t)(h.cap - 1);
  for (int64_t probe = 0; probe < h.cap; probe++) {
    unsigned long long prev = atomicCAS(&h.keys[s], EMPTY_KEY, key);
    if (prev == EMPTY_KEY || prev == key) return (int64_t)s;
    s = (s + 1) & (uint64_t)(h.cap - 1);
  }
  atomicOr(err, DEV_ERR_HASH_FULL);
  return -1;
}

__device__ int64_t hash_find(Hash h, unsigned long long key) {
  uint64_t s = mix64(key) & (uint64_t)(h.cap - 1);
  for (int64_t probe = 0; probe < h.cap; probe++) {
    unsigned long long k = h.keys[s];
    if (k == key) return (int64_t)s;
    if (k == EMPTY_KEY) return -1;
    s = (s + 1) & (uint64_t)(h.cap - 1);
  }
  return -1;
}

// ---------------------------------------------------------------------------
// mesh validation / index conversion
// ---------------------------------------------------------------------------
__global__ void k_to_zero_based(int32_t* a, int64_t n, int64_t nmax, uint32_t* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t v = a[i] - 1;
    if (v < 0 || v >= nmax) { atomicOr(err, DEV_ERR_NODE_RANGE); v = 0; }
    a[i] = v;
  }
}

// ---------------------------------------------------------------------------
// vertices
// ---------------------------------------------------------------------------
__global__ void k_fill_i32(int32_t* a, int64_t n, int32_t v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = v;
}
__global__ void k_corner_first(const int32_t* corners, int64_t nc, int32_t* first) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < nc) atomicMin(&first[corners[i]], (int32_t)i);
}
__global__ void k_corner_flags(const int32_t* corners, int64_t nc, const int32_t* first, int32_t* flag) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < nc) flag[i] = first[corners[i]] == (int32_t)i;
}
__global__ void k_noncorner_flags(const int32_t* first, int64_t nnodes, int32_t* flag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnodes; i += (int64_t)gridDim.x * blockDim.x)
    flag[i] = first[i] == INT_MAX;
}
__global__ void k_vertex_ids(const int32_t* corners, int64_t nc, const int32_t* first, const int32_t* cpos,
                             const int32_t* npos, int32_t ncu, int64_t nnodes, int32_t* node_vertex) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnodes; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t f = first[i];
    node_vertex[i] = f == INT_MAX ? ncu + npos[i] : cpos[f];
  }
}

// ---------------------------------------------------------------------------
// first-encounter face numbering
// ---------------------------------------------------------------------------
// instances: nf higher-dim faces, each with nlv vertices (fverts), nld local
// d-faces with ndv vertices given by ld (local vertex indices)
__global__ void k_insert_parents(Hash h, const int32_t* pverts, int64_t npar, int ndv, uint32_t* err) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= npar) return;
  int32_t v[4];
  for (int i = 0; i < ndv; i++) v[i] = pverts[p * ndv + i];
  int64_t s = hash_insert(h, face_key(v, ndv, err), err);
  if (s >= 0) h.vals[s] = (int32_t)(p + 1);
}
struct LocalFaces {
  int8_t v[12][4];
};
__global__ void k_insert_instances(Hash h, const int32_t* fverts, int64_t nf, int nlv, int nld, int ndv, LocalFaces ld,
                                   int64_t* inst_slot, uint32_t* err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nf * nld) return;
  int64_t f = r / nld;
  int l = (int)(r - f * nld);
  int32_t v[4];
  for (int i = 0; i < ndv; i++) v[i] = fverts[f * nlv + ld.v[l][i]];
  int64_t s = hash_insert(h, face_key(v, ndv, err), err);
  inst_slot[r] = s;
  if (s >= 0) atomicMin(&h.rank[s], (int32_t)r);
}
__global__ void k_first_flags(Hash h, int32_t* flag) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < h.cap; s += (int64_t)gridDim.x * blockDim.x)
    if (h.keys[s] != EMPTY_KEY && h.vals[s] == 0 && h.rank[s] != INT_MAX) flag[h.rank[s]] = 1;
}
__global__ void k_assign_new(Hash h, const int32_t* pos, int32_t npar) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < h.cap; s += (int64_t)gridDim.x * blockDim.x)
    if (h.keys[s] != EMPTY_KEY && h.vals[s] == 0 && h.rank[s] != INT_MAX) h.vals[s] = npar + pos[h.rank[s]] + 1;
}
__global__ void k_instance_ids(Hash h, const int64_t* inst_slot, int64_t n, int32_t* out, uint32_t* err) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = inst_slot[r];
    out[r] = s >= 0 ? h.vals[s] : 0;
    if (s < 0) atomicOr(err, DEV_ERR_LOOKUP);
  }
}
// vertices of every d-face: parents from their own list, new ones from the
// instance that first met them (generate_face_vertices, topology.jl:1468-1540)
__global__ void k_face_verts_parent(const int32_t* pverts, int64_t npar, int ndv, int32_t* dverts) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < npar * ndv) dverts[i] = pverts[i];
}
__global__ void k_face_verts_new(Hash h, int32_t npar, const int32_t* fverts, int nlv, int nld, int ndv,
                                 LocalFaces ld, int32_t* dverts) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < h.cap; s += (int64_t)gridDim.x * blockDim.x) {
    if (h.keys[s] == EMPTY_KEY) continue;
    int32_t id = h.vals[s];
    if (id <= npar) continue;
    int64_t r = h.rank[s];
    int64_t f = r / nld;
    int l = (int)(r - f * nld);
    for (int i = 0; i < ndv; i++) dverts[(int64_t)(id - 1) * ndv + i] = fverts[f * nlv + ld.v[l][i]];
  }
}
__global__ void k_lookup_instances(Hash h, const int32_t* fverts, int64_t nf, int nlv, int nld, int ndv, LocalFaces ld,
                                   int32_t* out, uint32_t* err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nf * nld) return;
  int64_t f = r / nld;
  int l = (int)(r - f * nld);
  int32_t v[4];
  for (int i = 0; i < ndv; i++) v[i] = fverts[f * nlv + ld.v[l][i]];
  int64_t s = hash_find(h, face_key(v, ndv, err));
  if (s < 0) { atomicOr(err, DEV_ERR_LOOKUP); out[r] = 0; } else out[r] = h.vals[s];
}

struct HashBuf {
  Hash h{};
  int alloc(Ctx* ctx, int64_t nkeys) {
    int64_t cap = 1024;
    while (cap < 2 * nkeys) cap <<= 1;
    h.cap = cap;
    GT_TRY(dalloc(ctx, &h.keys, cap));
    GT_TRY(dalloc(ctx, &h.vals, cap));
    GT_TRY(dalloc(ctx, &h.rank, cap));
    GT_CUDA(ctx, cudaMemsetAsync(h.keys, 0xFF, sizeof(unsigned long long) * cap, ctx->stream));
    GT_CUDA(ctx, cudaMemsetAsync(h.vals, 0, sizeof(int32_t) * cap, ctx->stream));
    k_fill_i32<<<GT_KC(ctx, grid_for(cap, 256)), 256, 0, ctx->stream>>>(h.rank, cap, INT_MAX);
    GT_LAUNCH(ctx, "k_fill_i32");
    return GT_OK;
  }
  void release(Ctx* ctx) {
    dfree(ctx, h.keys);
    dfree(ctx, h.vals);
    dfree(ctx, h.rank);
  }
};

// Numbers the d-faces of nf higher-dimensional faces (see file header).
// Outputs inst_ids[nf*nld] (1-based) and, if dverts != NULL, the vertices of
// every d-face (capacity npar + nf*nld faces).  Returns the count in *nd.
static int number_faces(Ctx* ctx, const int32_t* fverts, int64_t nf, int nlv, int nld, int ndv, const LocalFaces& ld,
                        const int32_t* pverts, int64_t npar, int32_t* inst_ids, int32_t** dverts_out, int64_t* nd) {
  HashBuf hb;
  int64_t ninst = nf * nld;
  int s = hb.alloc(ctx, npar + ninst);
  int64_t* inst_slot = nullptr;
  int32_t *flag = nullptr, *pos = nullptr;
  if (s == GT_OK) s = dalloc(ctx, &inst_slot, ninst);
  if (s == GT_OK) s = dalloc(ctx, &flag, ninst);
  if (s == GT_OK) s = dalloc(ctx, &pos, ninst + 1);
  if (s == GT_OK) {
    cudaStream_t st = ctx->stream;
    cudaMemsetAsync(flag, 0, sizeof(int32_t) * ninst, st);
    if (npar > 0) k_insert_parents<<<GT_KC(ctx, grid_for(npar, 256)), 256, 0, st>>>(hb.h, pverts, npar, ndv, ctx->d_err);
    k_insert_instances<<<GT_KC(ctx, grid_for(ninst, 256)), 256, 0, st>>>(hb.h, fverts, nf, nlv, nld, ndv, ld, inst_slot, ctx->d_err);
    k_first_flags<<<GT_KC(ctx, grid_for(hb.h.cap, 256)), 256, 0, st>>>(hb.h, flag);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) s = check_cuda(ctx, e, "face numbering");
  }
  if (s == GT_OK) s = exclusive_scan_i32(ctx, flag, pos, ninst);
  if (s == GT_OK) {
    cudaStream_t st = ctx->stream;
    k_assign_new<<<GT_KC(ctx, grid_for(hb.h.cap, 256)), 256, 0, st>>>(hb.h, pos, (int32_t)npar);
    k_instance_ids<<<GT_KC(ctx, grid_for(ninst, 256)), 256, 0, st>>>(hb.h, inst_slot, ninst, inst_ids, ctx->d_err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) s = check_cuda(ctx, e, "face ids");
  }
  if (s == GT_OK) {
    int32_t nnew = 0;
    cudaMemcpyAsync(&ctx->h_scratch[0], pos + ninst, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    memcpy(&nnew, &ctx->h_scratch[0], sizeof(int32_t));
    *nd = npar + nnew;
    if (dverts_out) {
      int32_t* dv = nullptr;
      s = dalloc(ctx, &dv, (*nd) * ndv);
      if (s == GT_OK) {
        cudaStream_t st = ctx->stream;
        if (npar > 0) k_face_verts_parent<<<GT_KC(ctx, grid_for(npar * ndv, 256)), 256, 0, st>>>(pverts, npar, ndv, dv);
        k_face_verts_new<<<GT_KC(ctx, grid_for(hb.h.cap, 256)), 256, 0, st>>>(hb.h, (int32_t)npar, fverts, nlv, nld, ndv, ld, dv);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) s = check_cuda(ctx, e, "face vertices");
        *dverts_out = dv;
      }
    }
  }
  dfree(ctx, inst_slot);
  dfree(ctx, flag);
  dfree(ctx, pos);
  hb.release(ctx);
  return s;
}

// lookup of existing d-faces (fill_face_boundary_mesh_topology!,
// src/topology.jl:515-591)
static int lookup_faces(Ctx* ctx, const int32_t* dverts, int64_t nd, int ndv, const int32_t* fverts, int64_t nf,
                        int nlv, int nld, const LocalFaces& ld, int32_t* out) {
  HashBuf hb;
  GT_TRY(hb.alloc(ctx, nd));
  cudaStream_t st = ctx->stream;
  k_insert_parents<<<GT_KC(ctx, grid_for(nd, 256)), 256, 0, st>>>(hb.h, dverts, nd, ndv, ctx->d_err);
  k_lookup_instances<<<GT_KC(ctx, grid_for(nf * nld, 256)), 256, 0, st>>>(hb.h, fverts, nf, nlv, nld, ndv, ld, out, ctx->d_err);
  cudaError_t e = cudaGetLastError();
  hb.release(ctx);
  if (e != cudaSuccess) return check_cuda(ctx, e, "face lookup");
  return GT_OK;
}

// ---------------------------------------------------------------------------
// DOF ids
// ---------------------------------------------------------------------------
__global__ void k_gather_cell_vertices(const int32_t* cell_nodes, int64_t n, const int32_t* node_vertex, int32_t* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = node_vertex[cell_nodes[i]] + 1;  // 1-based vertex ids
}

// global node-level dof (1-based, before the free/Dirichlet split):
// vertices, then edges, faces, cells (generate_dof_ids_step_1)
__global__ void k_cell_node_dofs(RefTables t, int order, int64_t nc, const int32_t* cverts, const int32_t* cedges,
                                 const int32_t* cfaces, int64_t nverts, int64_t nedges, int64_t nfaces,
                                 int32_t* cnd) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= nc) return;
  int32_t* o = cnd + c * t.nn;
  for (int v = 0; v < t.nlv; v++) o[t.vnode[v]] = cverts[c * t.nlv + v];
  if (order == 2) {
    for (int e = 0; e < t.nle; e++) o[t.enode[e]] = (int32_t)(nverts + cedges[c * t.nle + e]);
    if (t.face_nodes)
      for (int f = 0; f < 6; f++) o[t.fnode[f]] = (int32_t)(nverts + nedges + cfaces[c * 6 + f]);
    if (t.cell_node) o[t.cnode] = (int32_t)(nverts + nedges + nfaces + c + 1);
  }
}

// tag the closure nodes of tagged local (D-1)-faces (step_2, src/space.jl:487-508)
__global__ void k_tag_dirichlet(Hash tagged, RefTables t, int64_t nc, const int32_t* cverts, const int32_t* cnd,
                                int32_t* tag, uint32_t* err) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nc * t.nlf) return;
  int64_t c = r / t.nlf;
  int f = (int)(r - c * t.nlf);
  int32_t v[4];
  for (int i = 0; i < t.nlfv; i++) v[i] = cverts[c * t.nlv + t.lf_verts[f][i]];
  if (hash_find(tagged, face_key(v, t.nlfv, err)) < 0) return;
  for (int i = 0; i < t.nclosure; i++) tag[cnd[c * t.nn + t.closure[f][i]] - 1] = 1;
}
__global__ void k_free_flags(const int32_t* tag, int64_t n, int32_t* freef) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    freef[i] = 1 - tag[i];
}
__global__ void k_renumber(int32_t* cnd, int64_t n, const int32_t* tag, const int32_t* fpos, const int32_t* dpos) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t g = cnd[i] - 1;
    cnd[i] = tag[g] ? -(dpos[g] + 1) : fpos[g] + 1;
  }
}
__global__ void k_select_faces(const int32_t* bfaces, const int32_t* bgroup, int64_t nb, int nbfv, const int32_t* node_vertex,
                               const int32_t* groups, int ngroups, int32_t* out_verts, int32_t* keep) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nb) return;
  int k = 1;
  if (ngroups > 0) {
    k = 0;
    for (int g = 0; g < ngroups; g++) k |= bgroup[i] == groups[g];
  }
  keep[i] = k;
  for (int j = 0; j < nbfv; j++) out_verts[i * nbfv + j] = k ? node_vertex[bfaces[i * nbfv + j]] + 1 : 0;
}
__global__ void k_insert_tagged(Hash h, const int32_t* verts, const int32_t* keep, int64_t nb, int ndv, uint32_t* err) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nb || !keep[i]) return;
  hash_insert(h, face_key(verts + i * ndv, ndv, err), err);
}
__global__ void k_tag_vertices(const int32_t* sel, int64_t n, int32_t* tag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (sel[i] > 0) tag[sel[i] - 1] = 1;
}
__global__ void k_map_vertices(const int32_t* nodes, int64_t n, const int32_t* node_vertex, int32_t* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = node_vertex[nodes[i]] + 1;
}

static int device_error_status(Ctx* ctx, const char* where) {
  uint32_t bits = 0;
  GT_TRY(take_device_error(ctx, &bits));
  if (!bits) return GT_OK;
  std::string m = std::string(where) + ": ";
  if (bits & DEV_ERR_NODE_RANGE) m += "node id out of range; ";
  if (bits & DEV_ERR_KEY_RANGE) return set_error(ctx, GT_ERR_UNSUPPORTED, m + "more than 2^21-1 vertices for face keys");
  if (bits & DEV_ERR_HASH_FULL) m += "hash table full; ";
  if (bits & DEV_ERR_LOOKUP) m += "face not found (mesh is not a face complex); ";
  if (bits & DEV_ERR_ROW_CAP) m += "sparsity row above the supported width; ";
  return set_error(ctx, GT_ERR_INVALID, m);
}

// largest difference of two free node DOFs of one cell: per cell max - min,
// a warp maximum, one atomicMax per warp
__global__ void k_dof_spread(const int32_t* __restrict__ cnd, int64_t nc, int nn, int32_t* out) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int32_t v = 0;
  if (c < nc) {
    int32_t lo = INT_MAX, hi = 0;
    for (int a = 0; a < nn; a++) {
      const int32_t d = cnd[c * nn + a];
      if (d > 0) {
        lo = min(lo, d);
        hi = max(hi, d);
      }
    }
    if (hi > 0) v = hi - lo;
  }
  for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0 && v > 0) atomicMax(out, v);
}

int number_dofs(Space* sp, int ngroups, const int32_t* groups_host) {
  Mesh* M = sp->mesh;
  Ctx* ctx = M->ctx;
  cudaStream_t st = ctx->stream;
  RefTables t = make_ref_tables(M->ctype, sp->order);
  int64_t nc = M->ncells, nn_ = M->nnodes;
  int s = GT_OK;
  // ---- vertices
  int32_t *first = nullptr, *cflag = nullptr, *cpos = nullptr, *nflag = nullptr, *npos = nullptr, *node_vertex = nullptr;
  GT_TRY(dalloc(ctx, &first, nn_));
  GT_TRY(dalloc(ctx, &cflag, M->ncorners + 1));
  GT_TRY(dalloc(ctx, &cpos, M->ncorners + 1));
  GT_TRY(dalloc(ctx, &nflag, nn_));
  GT_TRY(dalloc(ctx, &npos, nn_ + 1));
  GT_TRY(dalloc(ctx, &node_vertex, nn_));
  k_fill_i32<<<GT_KC(ctx, grid_for(nn_, 256)), 256, 0, st>>>(first, nn_, INT_MAX);
  if (M->ncorners > 0) {
    k_corner_first<<<GT_KC(ctx, grid_for(M->ncorners, 256)), 256, 0, st>>>(M->corners, M->ncorners, first);
    k_corner_flags<<<GT_KC(ctx, grid_for(M->ncorners, 256)), 256, 0, st>>>(M->corners, M->ncorners, first, cflag);
  }
  k_noncorner_flags<<<GT_KC(ctx, grid_for(nn_, 256)), 256, 0, st>>>(first, nn_, nflag);
  GT_LAUNCH(ctx, "vertex flags");
  GT_TRY(exclusive_scan_i32(ctx, cflag, cpos, M->ncorners));
  GT_TRY(exclusive_scan_i32(ctx, nflag, npos, nn_));
  GT_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scratch[0], cpos + M->ncorners, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GT_CUDA(ctx, cudaStreamSynchronize(st));
  int32_t ncu = 0;
  memcpy(&ncu, &ctx->h_scratch[0], sizeof(int32_t));
  k_vertex_ids<<<GT_KC(ctx, grid_for(nn_, 256)), 256, 0, st>>>(M->corners, M->ncorners, first, cpos, npos, ncu, nn_, node_vertex);
  GT_LAUNCH(ctx, "k_vertex_ids");
  int64_t nverts = nn_;
  dfree(ctx, first);
  dfree(ctx, cflag);
  dfree(ctx, cpos);
  dfree(ctx, nflag);
  dfree(ctx, npos);
  // cell vertices (1-based vertex ids)
  int32_t* cverts = nullptr;
  GT_TRY(dalloc(ctx, &cverts, nc * M->nv));
  k_gather_cell_vertices<<<GT_KC(ctx, grid_for(nc * M->nv, 256)), 256, 0, st>>>(M->cell_nodes, nc * M->nv, node_vertex, cverts);
  GT_LAUNCH(ctx, "k_gather_cell_vertices");
  // ---- edges / faces (Q2)
  int32_t *cedges = nullptr, *cfaces = nullptr;
  int64_t nedges = 0, nfaces = 0;
  if (sp->order == 2) {
    LocalFaces lq{}, lh{}, le{};
    if (t.D == 2) {
      for (int e = 0; e < 4; e++) { lq.v[e][0] = t.le_verts[e][0]; lq.v[e][1] = t.le_verts[e][1]; }
      int32_t* pv = nullptr;
      GT_TRY(dalloc(ctx, &pv, M->nbfaces * 2));
      k_map_vertices<<<GT_KC(ctx, grid_for(M->nbfaces * 2, 256)), 256, 0, st>>>(M->bfaces, M->nbfaces * 2, node_vertex, pv);
      GT_LAUNCH(ctx, "k_map_vertices");
      GT_TRY(dalloc(ctx, &cedges, nc * 4));
      s = number_faces(ctx, cverts, nc, 4, 4, 2, lq, pv, M->nbfaces, cedges, nullptr, &nedges);
      dfree(ctx, pv);
      GT_TRY(s);
    } else if (M->ctype == GT_TET4) {
      // P2 tets: triangles numbered over the tets (parents: the boundary
      // triangles), edges over the triangles (parents: the boundary 1-faces),
      // then each tet's 6 edges looked up (create_face_boundary!,
      // src/topology.jl:1099-1125, generates d-faces from the (d+1)-faces)
      LocalFaces ltf{}, ltri{}, lte{};
      for (int f = 0; f < 4; f++)
        for (int i = 0; i < 3; i++) ltf.v[f][i] = t.lf_verts[f][i];
      static const int TRE[3][2] = {{0, 1}, {0, 2}, {1, 2}};  // edges of the unit triangle, src/domain.jl:413-424
      for (int e = 0; e < 3; e++) { ltri.v[e][0] = TRE[e][0]; ltri.v[e][1] = TRE[e][1]; }
      for (int e = 0; e < 6; e++) { lte.v[e][0] = t.le_verts[e][0]; lte.v[e][1] = t.le_verts[e][1]; }
      int32_t *pf = nullptr, *pe = nullptr, *fverts = nullptr, *fedges = nullptr, *everts = nullptr;
      GT_TRY(dalloc(ctx, &pf, M->nbfaces * 3 + 1));
      GT_TRY(dalloc(ctx, &pe, M->nbedges * 2 + 1));
      if (M->nbfaces > 0)
        k_map_vertices<<<GT_KC(ctx, grid_for(M->nbfaces * 3, 256)), 256, 0, st>>>(M->bfaces, M->nbfaces * 3, node_vertex, pf);
      if (M->nbedges > 0)
        k_map_vertices<<<GT_KC(ctx, grid_for(M->nbedges * 2, 256)), 256, 0, st>>>(M->bedges, M->nbedges * 2, node_vertex, pe);
      GT_LAUNCH(ctx, "k_map_vertices");
      GT_TRY(dalloc(ctx, &cfaces, nc * 4));
      GT_TRY(number_faces(ctx, cverts, nc, 4, 4, 3, ltf, pf, M->nbfaces, cfaces, &fverts, &nfaces));
      GT_TRY(dalloc(ctx, &fedges, nfaces * 3));
      GT_TRY(number_faces(ctx, fverts, nfaces, 3, 3, 2, ltri, pe, M->nbedges, fedges, &everts, &nedges));
      GT_TRY(dalloc(ctx, &cedges, nc * 6));
      GT_TRY(lookup_faces(ctx, everts, nedges, 2, cverts, nc, 4, 6, lte, cedges));
      dfree(ctx, pf);
      dfree(ctx, pe);
      dfree(ctx, fverts);
      dfree(ctx, fedges);
      dfree(ctx, everts);
    } else {
      for (int f = 0; f < 6; f++)
        for (int i = 0; i < 4; i++) lh.v[f][i] = t.lf_verts[f][i];
      static const int QE[4][2] = {{0, 1}, {2, 3}, {0, 2}, {1, 3}};
      for (int e = 0; e < 4; e++) { lq.v[e][0] = QE[e][0]; lq.v[e][1] = QE[e][1]; }
      for (int e = 0; e < 12; e++) { le.v[e][0] = t.le_verts[e][0]; le.v[e][1] = t.le_verts[e][1]; }
      int32_t *pf = nullptr, *pe = nullptr, *fverts = nullptr, *fedges = nullptr, *everts = nullptr;
      GT_TRY(dalloc(ctx, &pf, M->nbfaces * 4));
      GT_TRY(dalloc(ctx, &pe, M->nbedges * 2 + 1));
      k_map_vertices<<<GT_KC(ctx, grid_for(M->nbfaces * 4, 256)), 256, 0, st>>>(M->bfaces, M->nbfaces * 4, node_vertex, pf);
      if (M->nbedges > 0)
        k_map_vertices<<<GT_KC(ctx, grid_for(M->nbedges * 2, 256)), 256, 0, st>>>(M->bedges, M->nbedges * 2, node_vertex, pe);
      GT_LAUNCH(ctx, "k_map_vertices");
      GT_TRY(dalloc(ctx, &cfaces, nc * 6));
      GT_TRY(number_faces(ctx, cverts, nc, 8, 6, 4, lh, pf, M->nbfaces, cfaces, &fverts, &nfaces));
      GT_TRY(dalloc(ctx, &fedges, nfaces * 4));
      GT_TRY(number_faces(ctx, fverts, nfaces, 4, 4, 2, lq, pe, M->nbedges, fedges, &everts, &nedges));
      GT_TRY(dalloc(ctx, &cedges, nc * 12));
      GT_TRY(lookup_faces(ctx, everts, nedges, 2, cverts, nc, 8, 12, le, cedges));
      dfree(ctx, pf);
      dfree(ctx, pe);
      dfree(ctx, fverts);
      dfree(ctx, fedges);
      dfree(ctx, everts);
    }
  }
  // ---- node dofs before the split
  // node dofs: vertices, then (order 2) edges, 2-faces and cells that own a node
  if (!t.face_nodes) nfaces = 0;
  int64_t nnodes_sp = nverts + (sp->order == 2 ? nedges + nfaces + (t.cell_node ? nc : 0) : 0);
  GT_TRY(dalloc(ctx, &sp->cell_ndofs, nc * t.nn));
  k_cell_node_dofs<<<GT_KC(ctx, grid_for(nc, 128)), 128, 0, st>>>(t, sp->order, nc, cverts, cedges, cfaces, nverts, nedges, nfaces,
                                                       sp->cell_ndofs);
  GT_LAUNCH(ctx, "k_cell_node_dofs");
  // ---- Dirichlet tags
  int32_t *tag = nullptr, *freef = nullptr, *fpos = nullptr, *dpos = nullptr;
  GT_TRY(dalloc(ctx, &tag, nnodes_sp));
  GT_CUDA(ctx, cudaMemsetAsync(tag, 0, sizeof(int32_t) * nnodes_sp, st));
  if (ngroups != 0 && M->nbfaces > 0) {
    int32_t *sel = nullptr, *keep = nullptr, *dgroups = nullptr;
    int ng = ngroups > 0 ? ngroups : 0;
    GT_TRY(dalloc(ctx, &sel, M->nbfaces * M->nbfv));
    GT_TRY(dalloc(ctx, &keep, M->nbfaces));
    GT_TRY(dalloc(ctx, &dgroups, ng + 1));
    if (ng > 0) GT_TRY(copy_in(ctx, dgroups, groups_host, ng));
    k_select_faces<<<GT_KC(ctx, grid_for(M->nbfaces, 256)), 256, 0, st>>>(M->bfaces, M->bgroup, M->nbfaces, M->nbfv, node_vertex,
                                                               dgroups, ng, sel, keep);
    GT_LAUNCH(ctx, "k_select_faces");
    if (sp->order == 1) {
      // the closure of a tagged face holds only its vertices, whose
      // pre-split node dof is the vertex id
      k_tag_vertices<<<GT_KC(ctx, grid_for(M->nbfaces * M->nbfv, 256)), 256, 0, st>>>(sel, M->nbfaces * M->nbfv, tag);
      GT_LAUNCH(ctx, "k_tag_vertices");
    } else {
      HashBuf hb;
      GT_TRY(hb.alloc(ctx, M->nbfaces));
      k_insert_tagged<<<GT_KC(ctx, grid_for(M->nbfaces, 256)), 256, 0, st>>>(hb.h, sel, keep, M->nbfaces, M->nbfv, ctx->d_err);
      k_tag_dirichlet<<<GT_KC(ctx, grid_for(nc * t.nlf, 256)), 256, 0, st>>>(hb.h, t, nc, cverts, sp->cell_ndofs, tag, ctx->d_err);
      GT_LAUNCH(ctx, "k_tag_dirichlet");
      hb.release(ctx);
    }
    dfree(ctx, sel);
    dfree(ctx, keep);
    dfree(ctx, dgroups);
  }
  GT_TRY(dalloc(ctx, &freef, nnodes_sp));
  GT_TRY(dalloc(ctx, &fpos, nnodes_sp + 1));
  GT_TRY(dalloc(ctx, &dpos, nnodes_sp + 1));
  k_free_flags<<<GT_KC(ctx, grid_for(nnodes_sp, 256)), 256, 0, st>>>(tag, nnodes_sp, freef);
  GT_LAUNCH(ctx, "k_free_flags");
  GT_TRY(exclusive_scan_i32(ctx, freef, fpos, nnodes_sp));
  GT_TRY(exclusive_scan_i32(ctx, tag, dpos, nnodes_sp));
  k_renumber<<<GT_KC(ctx, grid_for(nc * t.nn, 256)), 256, 0, st>>>(sp->cell_ndofs, nc * t.nn, tag, fpos, dpos);
  GT_LAUNCH(ctx, "k_renumber");
  GT_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scratch[0], fpos + nnodes_sp, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GT_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scratch[1], dpos + nnodes_sp, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  int32_t* dspread = nullptr;
  GT_TRY(dalloc(ctx, &dspread, 1));
  GT_CUDA(ctx, cudaMemsetAsync(dspread, 0, sizeof(int32_t), st));
  if (nc > 0) k_dof_spread<<<GT_KC(ctx, grid_for(nc, 256)), 256, 0, st>>>(sp->cell_ndofs, nc, t.nn, dspread);
  GT_LAUNCH(ctx, "k_dof_spread");
  GT_CUDA(ctx, cudaMemcpyAsync(&ctx->h_scratch[2], dspread, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  const int ds = device_error_status(ctx, "lagrange_space");  // synchronises
  dfree(ctx, dspread);
  GT_TRY(ds);
  int32_t nf = 0, ndr = 0, spread = 0;
  memcpy(&nf, &ctx->h_scratch[0], sizeof(int32_t));
  memcpy(&ndr, &ctx->h_scratch[1], sizeof(int32_t));
  memcpy(&spread, &ctx->h_scratch[2], sizeof(int32_t));
  sp->nfree_nodes = nf;
  sp->ndiri_nodes = ndr;
  sp->dof_spread = spread;
  dfree(ctx, tag);
  dfree(ctx, freef);
  dfree(ctx, fpos);
  dfree(ctx, dpos);
  dfree(ctx, cverts);
  dfree(ctx, cedges);
  dfree(ctx, cfaces);
  dfree(ctx, node_vertex);
  return GT_OK;
}

__global__ void k_expand_cell_dofs(const int32_t* cnd, int64_t nc, int nn, int ncomp, int32_t* out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nc * nn * ncomp) return;
  int64_t c = i / (nn * ncomp);
  int r = (int)(i - c * nn * ncomp);
  int a = r / ncomp, k = r - a * ncomp;
  int32_t d = cnd[c * nn + a];
  out[i] = d > 0 ? (d - 1) * ncomp + k + 1 : -((-d - 1) * ncomp + k + 1);
}

// ---------------------------------------------------------------------------
// Boundary integrals: GT.assemble_vector(v -> int g v dGamma) over boundary
// faces of given groups (the Neumann term of docs/src/src_jl/
// example_poisson_equation.jl:161-203; src/problems.jl:244-274 with a
// boundary measure).  The selected boundary faces are found as local faces
// of their cells (hash of the sorted node ids), listed in (cell, local face)
// order; each gets its face vector over the closure nodes of the face
// (Gauss points with order + 1 per direction on quadrilateral faces and
// edges, the 3-point degree-2 rule on triangles; dGamma = |dx/ds| or
// |dx/ds x dx/dt| dS); and every free DOF sums its face contributions in
// that order (incidence lists, as for the cell scatter).
// ---------------------------------------------------------------------------
__global__ void k_insert_bfaces(Hash h, const int32_t* bfaces, const int32_t* bgroup, int64_t nb, int nbfv,
                                const int32_t* groups, int ngroups, uint32_t* err) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nb) return;
  if (ngroups > 0) {
    int k = 0;
    for (int g = 0; g < ngroups; g++) k |= bgroup[i] == groups[g];
    if (!k) return;
  }
  hash_insert(h, face_key(bfaces + i * nbfv, nbfv, err), err);
}

__global__ void k_flag_bfaces(Hash h, RefTables t, int64_t nc, const int32_t* cell_nodes, int32_t* flag, uint32_t* err) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nc * t.nlf) return;
  const int64_t c = r / t.nlf;
  const int f = (int)(r - c * t.nlf);
  int32_t v[4];
  for (int i = 0; i < t.nlfv; i++) v[i] = cell_nodes[c * t.nlv + t.lf_verts[f][i]];
  flag[r] = hash_find(h, face_key(v, t.nlfv, err)) >= 0 ? 1 : 0;
}

__global__ void k_compact_bfaces(const int32_t* flag, const int32_t* pos, int64_t n, int32_t* list) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r < n && flag[r]) list[pos[r]] = (int32_t)r;
}

__device__ __forceinline__ double lagr(int order, int e, double x) {
  if (order == 1) return e == 0 ? 1.0 - x : x;
  return e == 0 ? 2.0 * (x - 0.5) * (x - 1.0) : (e == 1 ? -4.0 * x * (x - 1.0) : 2.0 * x * (x - 0.5));
}

// one thread per selected face: fe[(j * ncl + i) * ncomp + k] = g_k int phi_i
// dGamma over the closure node i of face j; fdofs[j * ncl + i] its node DOF
__global__ void k_face_vectors(const int32_t* list, int64_t nsel, RefTables t, int ctype, int order,
                               const double* coords, const int32_t* cell_nodes, const int32_t* cnd, const double* g,
                               int ncomp, double* fe, int32_t* fdofs) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= nsel) return;
  const int64_t id = list[j], c = id / t.nlf;
  const int f = (int)(id - c * t.nlf), D = t.D, ncl = t.nclosure;
  double X[8][3];
  for (int v = 0; v < t.nlv; v++)
    for (int d = 0; d < 3; d++) X[v][d] = d < D ? coords[(int64_t)cell_nodes[c * t.nlv + v] * D + d] : 0.0;
  double acc[9];
  for (int i = 0; i < ncl; i++) {
    acc[i] = 0.0;
    fdofs[j * ncl + i] = cnd[c * t.nn + t.closure[f][i]];
  }
  if (ctype == GT_TET4) {
    // a flat triangle: the 3-point degree-2 rule at face-barycentric
    // (2/3, 1/6, 1/6) and permutations, weights 1/6 on the unit right
    // triangle; the cell's basis (P1: barycentric l_i; P2: l_i (2 l_i - 1) at
    // the vertex nodes 0, 2, 5, 9 and 4 l_i l_j at the edge nodes) at the
    // point's cell-barycentric coordinates
    const int a0 = t.lf_verts[f][0], a1 = t.lf_verts[f][1], a2 = t.lf_verts[f][2];
    double e1[3], e2[3], n[3];
    for (int d = 0; d < 3; d++) { e1[d] = X[a1][d] - X[a0][d]; e2[d] = X[a2][d] - X[a0][d]; }
    n[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const double jac = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int q = 0; q < 3; q++) {
      double l[4] = {0, 0, 0, 0};
      for (int i = 0; i < 3; i++) l[t.lf_verts[f][i]] = i == q ? 2.0 / 3.0 : 1.0 / 6.0;
      double phi[10];
      if (order == 1) {
        for (int i = 0; i < 4; i++) phi[i] = l[i];
      } else {
        const int vi[4] = {0, 2, 5, 9};
        const int ep[6][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}}, en[6] = {1, 3, 4, 6, 7, 8};
        for (int i = 0; i < 4; i++) phi[vi[i]] = l[i] * (2.0 * l[i] - 1.0);
        for (int e = 0; e < 6; e++) phi[en[e]] = 4.0 * l[ep[e][0]] * l[ep[e][1]];
      }
      for (int i = 0; i < ncl; i++) acc[i] += (1.0 / 6.0) * jac * phi[t.closure[f][i]];
    }
  } else {
    const int dir = D == 2 ? (f < 2 ? 1 : 0) : 2 - f / 2, side = f & 1;
    int fr[2], nfr = 0;
    for (int d = 0; d < D; d++)
      if (d != dir) fr[nfr++] = d;
    const int n1 = order + 1, m = order + 1;
    double gp[3], gw[3];
    if (n1 == 2) {
      const double s = 0.5 / sqrt(3.0);
      gp[0] = 0.5 - s; gp[1] = 0.5 + s; gw[0] = gw[1] = 0.5;
    } else {
      const double s = 0.5 * sqrt(0.6);
      gp[0] = 0.5 - s; gp[1] = 0.5; gp[2] = 0.5 + s;
      gw[0] = 5.0 / 18.0; gw[1] = 8.0 / 18.0; gw[2] = 5.0 / 18.0;
    }
    const int nq = D == 2 ? n1 : n1 * n1;
    for (int q = 0; q < nq; q++) {
      double xi[3] = {0, 0, 0};
      xi[dir] = (double)side;
      xi[fr[0]] = gp[q % n1];
      double w = gw[q % n1];
      if (D == 3) {
        xi[fr[1]] = gp[q / n1];
        w *= gw[q / n1];
      }
      // tangents dx/dxi_a of the multilinear geometry map
      double tg[2][3] = {{0, 0, 0}, {0, 0, 0}};
      for (int v = 0; v < t.nlv; v++) {
        for (int a = 0; a < nfr; a++) {
          double dn = 1.0;
          for (int d = 0; d < D; d++) {
            const int bit = (v >> d) & 1;
            dn *= d == fr[a] ? (bit ? 1.0 : -1.0) : (bit ? xi[d] : 1.0 - xi[d]);
          }
          for (int d = 0; d < D; d++) tg[a][d] += X[v][d] * dn;
        }
      }
      double jac;
      if (D == 2) {
        jac = sqrt(tg[0][0] * tg[0][0] + tg[0][1] * tg[0][1]);
      } else {
        const double cx = tg[0][1] * tg[1][2] - tg[0][2] * tg[1][1], cy = tg[0][2] * tg[1][0] - tg[0][0] * tg[1][2],
                     cz = tg[0][0] * tg[1][1] - tg[0][1] * tg[1][0];
        jac = sqrt(cx * cx + cy * cy + cz * cz);
      }
      for (int i = 0; i < ncl; i++) {
        const int k = t.closure[f][i];
        const int e[3] = {k % m, (k / m) % m, k / (m * m)};
        double phi = 1.0;
        for (int d = 0; d < D; d++) phi *= lagr(order, e[d], xi[d]);
        acc[i] += w * jac * phi;
      }
    }
  }
  for (int i = 0; i < ncl; i++)
    for (int k = 0; k < ncomp; k++) fe[(j * ncl + i) * ncomp + k] = g[k] * acc[i];
}

// b[r] (+)= the face contributions of free node r, in (cell, local face) order
__global__ void k_gather_bvec(const int64_t* inc_ptr, const int32_t* inc, int64_t nrows, const double* fe, int ncomp,
                              double* b, int accumulate) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  for (int k = 0; k < ncomp; k++) {
    double s = 0.0;
    for (int64_t e = inc_ptr[r]; e < inc_ptr[r + 1]; e++) s += fe[(int64_t)inc[e] * ncomp + k];
    b[r * ncomp + k] = accumulate ? b[r * ncomp + k] + s : s;
  }
}

}  // namespace gt

using namespace gt;

extern "C" {

int gt_mesh_create(gt_ctx* ctx, int cell_type, int64_t nnodes, const double* coords, int64_t ncells,
                   const int32_t* cell_nodes, int64_t ncorners, const int32_t* corner_nodes, int64_t nbfaces,
                   const int32_t* bface_nodes, const int32_t* bface_group, int64_t nbedges, const int32_t* bedge_nodes,
                   gt_mesh** out) {
  if (!ctx || !out) return GT_ERR_INVALID;
  *out = nullptr;
  if (cell_type != GT_QUAD4 && cell_type != GT_HEX8 && cell_type != GT_TET4)
    return set_error(ctx, GT_ERR_UNSUPPORTED, "cell type must be QUAD4, HEX8 or TET4");
  if (nnodes <= 0 || ncells <= 0 || !coords || !cell_nodes) return set_error(ctx, GT_ERR_INVALID, "empty mesh");
  if (nnodes >= INT_MAX || ncells >= INT_MAX / 8) return set_error(ctx, GT_ERR_UNSUPPORTED, "mesh too large for Int32 ids");
  cudaSetDevice(ctx->device);
  gt_mesh* M = new gt_mesh();
  M->ctx = ctx;
  M->ctype = cell_type;
  M->D = cell_type == GT_QUAD4 ? 2 : 3;
  M->nv = cell_type == GT_QUAD4 ? 4 : (cell_type == GT_HEX8 ? 8 : 4);
  M->nbfv = cell_type == GT_QUAD4 ? 2 : (cell_type == GT_HEX8 ? 4 : 3);
  M->nnodes = nnodes;
  M->ncells = ncells;
  M->ncorners = ncorners;
  M->nbfaces = nbfaces;
  M->nbedges = M->D == 3 ? nbedges : 0;
  int s = GT_OK;
  auto up = [&](int32_t** dst, const int32_t* src, int64_t n, int64_t nmax) {
    if (s != GT_OK) return;
    s = dalloc(ctx, dst, n > 0 ? n : 1);
    if (s != GT_OK || n <= 0) return;
    s = copy_in(ctx, *dst, src, n);
    if (s != GT_OK) return;
    if (nmax > 0) k_to_zero_based<<<GT_KC(ctx, grid_for(n, 256)), 256, 0, ctx->stream>>>(*dst, n, nmax, ctx->d_err);
  };
  s = dalloc(ctx, &M->coords, nnodes * M->D);
  if (s == GT_OK) s = copy_in(ctx, M->coords, coords, nnodes * M->D);
  up(&M->cell_nodes, cell_nodes, ncells * M->nv, nnodes);
  up(&M->corners, corner_nodes, ncorners, nnodes);
  up(&M->bfaces, bface_nodes, nbfaces * M->nbfv, nnodes);
  up(&M->bgroup, bface_group, bface_group ? nbfaces : 0, 0);
  up(&M->bedges, bedge_nodes, M->nbedges * 2, nnodes);
  if (s == GT_OK) s = device_error_status(ctx, "gt_mesh_create");
  if (s != GT_OK) {
    gt_mesh_destroy(M);
    return s;
  }
  *out = M;
  return GT_OK;
}

int gt_mesh_set_coords(gt_mesh* M, const double* coords) {
  if (!M || !coords) return GT_ERR_INVALID;
  Ctx* ctx = M->ctx;
  cudaPointerAttributes at{};
  bool dev = cudaPointerGetAttributes(&at, coords) == cudaSuccess &&
             (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged);
  cudaGetLastError();
  if (dev) return copy_in(ctx, M->coords, coords, M->nnodes * M->D);
  // host source: uploaded on the copy stream, overlapping whatever the next
  // call runs before it needs coordinates (numbering, sparsity)
  cudaEvent_t ev = nullptr;
  GT_TRY(side_copy_in(ctx, M->coords, coords, sizeof(double) * M->nnodes * M->D, &ev));
  if (M->coords_ev) event_put(ctx, M->coords_ev);
  M->coords_ev = ev;
  M->coords_pending = true;
  return GT_OK;
}

int gt_mesh_destroy(gt_mesh* M) {
  if (!M) return GT_ERR_INVALID;
  Ctx* c = M->ctx;
  mesh_wait_coords(M);  // no upload may still target the freed buffer
  if (M->coords_ev) event_put(c, M->coords_ev);
  dfree(c, M->coords);
  dfree(c, M->cell_nodes);
  dfree(c, M->corners);
  dfree(c, M->bfaces);
  dfree(c, M->bgroup);
  dfree(c, M->bedges);
  delete M;
  return GT_OK;
}

int gt_space_create(gt_mesh* M, int order, int ncomp, int ngroups, const int32_t* groups, gt_space** out) {
  if (!M || !out) return GT_ERR_INVALID;
  *out = nullptr;
  Ctx* ctx = M->ctx;
  if (order != 1 && order != 2) return set_error(ctx, GT_ERR_UNSUPPORTED, "order must be 1 or 2");
  if (ncomp != 1 && ncomp != M->D) return set_error(ctx, GT_ERR_UNSUPPORTED, "ncomp must be 1 or the dimension");
  if (ngroups > 0 && !groups) return set_error(ctx, GT_ERR_INVALID, "groups is NULL");
  if (ngroups != 0 && M->nbfaces > 0 && M->ctype == GT_QUAD4 && !M->bgroup && ngroups > 0)
    return set_error(ctx, GT_ERR_INVALID, "mesh has no boundary groups");
  cudaSetDevice(ctx->device);
  gt_space* sp = new gt_space();
  sp->ctx = ctx;
  sp->mesh = M;
  sp->order = order;
  sp->ncomp = ncomp;
  sp->nn = space_nodes(M->ctype, order);
  sp->nloc = sp->nn * ncomp;
  int s = number_dofs(sp, ngroups, groups);
  if (s != GT_OK) {
    gt_space_destroy(sp);
    return s;
  }
  *out = sp;
  return GT_OK;
}

int gt_space_info(const gt_space* sp, int64_t* info) {
  if (!sp || !info) return GT_ERR_INVALID;
  info[0] = sp->nfree_nodes * sp->ncomp;
  info[1] = sp->ndiri_nodes * sp->ncomp;
  info[2] = sp->nloc;
  info[3] = sp->mesh->ncells;
  info[4] = sp->nfree_nodes;
  info[5] = sp->ncomp;
  return GT_OK;
}

int gt_space_cell_dofs(const gt_space* sp, int32_t* out) {
  if (!sp || !out) return GT_ERR_INVALID;
  Ctx* ctx = sp->mesh->ctx;
  int64_t n = sp->mesh->ncells * sp->nloc;
  int32_t* tmp = nullptr;
  GT_TRY(dalloc(ctx, &tmp, n));
  k_expand_cell_dofs<<<GT_KC(ctx, grid_for(n, 256)), 256, 0, ctx->stream>>>(sp->cell_ndofs, sp->mesh->ncells, sp->nn, sp->ncomp, tmp);
  GT_LAUNCH(ctx, "k_expand_cell_dofs");
  int s = copy_out(ctx, out, tmp, n);
  if (s == GT_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) s = check_cuda(ctx, e, "gt_space_cell_dofs");
  }
  dfree(ctx, tmp);
  return s;
}

int gt_assemble_boundary_vector(gt_space* sp, int ngroups, const int32_t* groups, const double* g, double* b,
                                int accumulate) {
  if (!sp || !g || !b) return GT_ERR_INVALID;
  Ctx* ctx = sp->mesh->ctx;
  Mesh* M = sp->mesh;
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  const RefTables t = make_ref_tables(M->ctype, sp->order);
  const int64_t nc = M->ncells, nflag = nc * t.nlf, nb = sp->nfree_nodes * sp->ncomp;
  const bool dev_b = [&] {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, b) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
  }();
  double* bd = b;
  if (!dev_b) {
    GT_TRY(dalloc(ctx, &bd, nb > 0 ? nb : 1));
    if (accumulate && nb > 0) GT_TRY(copy_in(ctx, bd, b, nb));
  }
  int32_t *dgroups = nullptr, *flag = nullptr, *pos = nullptr, *list = nullptr, *fdofs = nullptr, *inc = nullptr;
  double *dg = nullptr, *fe = nullptr;
  int64_t* inc_ptr = nullptr;
  int64_t nsel = 0, ninc = 0;
  const int ng = ngroups > 0 ? ngroups : 0;
  mesh_wait_coords(M);
  int s = dalloc(ctx, &dgroups, ng + 1);
  if (s == GT_OK && ng > 0) s = copy_in(ctx, dgroups, groups, ng);
  if (s == GT_OK) s = dalloc(ctx, &dg, sp->ncomp);
  if (s == GT_OK) s = copy_in(ctx, dg, g, sp->ncomp);
  if (s == GT_OK) s = dalloc(ctx, &flag, nflag + 1);
  if (s == GT_OK) s = dalloc(ctx, &pos, nflag + 1);
  if (s == GT_OK && M->nbfaces > 0 && nflag > 0) {
    HashBuf hb;
    s = hb.alloc(ctx, M->nbfaces);
    if (s == GT_OK) {
      k_insert_bfaces<<<GT_KC(ctx, grid_for(M->nbfaces, 256)), 256, 0, st>>>(hb.h, M->bfaces, M->bgroup, M->nbfaces,
                                                                             M->nbfv, dgroups, ng, ctx->d_err);
      k_flag_bfaces<<<GT_KC(ctx, grid_for(nflag, 256)), 256, 0, st>>>(hb.h, t, nc, M->cell_nodes, flag, ctx->d_err);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) s = check_cuda(ctx, e, "k_flag_bfaces");
    }
    if (s == GT_OK) s = exclusive_scan_i32(ctx, flag, pos, nflag);
    if (s == GT_OK) {
      int32_t tot = 0;
      s = copy_out(ctx, &tot, pos + nflag, 1);
      if (s == GT_OK) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) s = check_cuda(ctx, e, "boundary faces");
      }
      nsel = tot;
    }
    hb.release(ctx);
  }
  if (s == GT_OK && nsel > 0) {
    s = dalloc(ctx, &list, nsel);
    if (s == GT_OK) s = dalloc(ctx, &fdofs, nsel * t.nclosure);
    if (s == GT_OK) s = dalloc(ctx, &fe, nsel * t.nclosure * sp->ncomp);
    if (s == GT_OK) {
      k_compact_bfaces<<<GT_KC(ctx, grid_for(nflag, 256)), 256, 0, st>>>(flag, pos, nflag, list);
      k_face_vectors<<<GT_KC(ctx, grid_for(nsel, 128)), 128, 0, st>>>(list, nsel, t, M->ctype, sp->order, M->coords,
                                                                      M->cell_nodes, sp->cell_ndofs, dg, sp->ncomp, fe,
                                                                      fdofs);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) s = check_cuda(ctx, e, "k_face_vectors");
    }
    if (s == GT_OK) s = build_incidence_arr(ctx, fdofs, nsel * t.nclosure, sp->nfree_nodes, &inc_ptr, &inc, &ninc, true);
  }
  if (s == GT_OK && sp->nfree_nodes > 0) {
    if (nsel > 0) {
      k_gather_bvec<<<GT_KC(ctx, grid_for(sp->nfree_nodes, 256)), 256, 0, st>>>(inc_ptr, inc, sp->nfree_nodes, fe,
                                                                                sp->ncomp, bd, accumulate);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) s = check_cuda(ctx, e, "k_gather_bvec");
    } else if (!accumulate) {
      cudaError_t e = cudaMemsetAsync(bd, 0, sizeof(double) * nb, st);
      if (e != cudaSuccess) s = check_cuda(ctx, e, "memset");
    }
  }
  if (s == GT_OK && !dev_b && nb > 0) s = copy_out(ctx, b, bd, nb);
  if (s == GT_OK) s = device_error_status(ctx, "assemble_boundary_vector");  // synchronises
  if (!dev_b) dfree(ctx, bd);
  dfree(ctx, dgroups);
  dfree(ctx, dg);
  dfree(ctx, flag);
  dfree(ctx, pos);
  dfree(ctx, list);
  dfree(ctx, fdofs);
  dfree(ctx, fe);
  dfree(ctx, inc_ptr);
  dfree(ctx, inc);
  return s;
}

int gt_space_destroy(gt_space* sp) {
  if (!sp) return GT_ERR_INVALID;
  Ctx* c = sp->ctx;
  dfree(c, sp->cell_ndofs);
  dfree(c, sp->inc_ptr);
  dfree(c, sp->inc);
  delete sp;
  return GT_OK;
}

}  // extern "C"
