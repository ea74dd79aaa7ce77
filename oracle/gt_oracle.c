/*
 * gt_oracle.c -- CPU restatement of GalerkinToolkit.jl's finite-element
 * assembly path (mesh generation, topology numbering, DOF ids, quadrature,
 * per-cell integration, COO append and COO->CSC compression, plus a Jacobi
 * preconditioned CG used as the solve checker).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle and the
 * timed CPU baseline.  Nothing in the product library links or calls it.
 *
 * Every function cites the reference file:line (paths inside the
 * GalerkinToolkit.jl v0.6.3 source tree) whose algorithm it restates.
 * Loops keep the reference's iteration order wherever the order decides a
 * result (face numbering by first encounter, COO append order, the order in
 * which duplicate COO entries are summed).
 *
 * Conventions (the reference's, src/helpers.jl:47-61): node, vertex, face
 * and cell ids are 1-based Int32; DOF ids are 1-based for free DOFs and
 * negative for Dirichlet DOFs (src/space.jl:515-524).  CSC/CSR outputs are
 * 0-based (ptr arrays int64, index arrays int32).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Reference-cell tables                                                     */
/* ------------------------------------------------------------------------ */

/* Unit square / cube local faces, src/domain.jl:222-223 and :251-258. */
static const int QUAD_EDGES[4][2] = {{1, 2}, {3, 4}, {1, 3}, {2, 4}};
static const int HEX_EDGES[12][2] = {{1, 2}, {3, 4}, {1, 3}, {2, 4}, {5, 6}, {7, 8},
                                     {5, 7}, {6, 8}, {1, 5}, {3, 7}, {2, 6}, {4, 8}};
static const int HEX_FACES[6][4] = {{1, 2, 3, 4}, {5, 6, 7, 8}, {1, 2, 5, 6},
                                    {3, 4, 7, 8}, {1, 3, 5, 7}, {2, 4, 6, 8}};
/* Unit tetrahedron local faces, src/domain.jl:451-456. */
static const int TET_FACES[4][3] = {{1, 2, 3}, {1, 2, 4}, {1, 3, 4}, {2, 3, 4}};
/* Six-tetrahedra split of the unit cube, src/domain.jl:333-336. */
static const int CUBE_TETS[6][4] = {{1, 2, 3, 7}, {1, 2, 5, 7}, {2, 3, 4, 7},
                                    {2, 4, 7, 8}, {2, 5, 6, 7}, {2, 6, 7, 8}};

enum { OR_QUAD4 = 1, OR_HEX8 = 2, OR_TET4 = 3 };
enum { OR_LAPLACE = 1, OR_MASS = 2, OR_ELASTICITY = 3 };

/* ------------------------------------------------------------------------ */
/* Seeded synthetic inputs: splitmix64 keyed draws                           */
/* ------------------------------------------------------------------------ */

static uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  uint64_t z = x;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
double or_uniform(uint64_t seed, uint64_t key) {
  return (double)(splitmix64(seed ^ key) >> 11) * (1.0 / 9007199254740992.0);
}

/* ------------------------------------------------------------------------ */
/* Small open-addressing map: sorted vertex tuple (<=4 ids) -> int32 value   */
/* ------------------------------------------------------------------------ */

typedef struct {
  int64_t cap;
  int32_t* keys; /* cap * 4, 0 = empty */
  int32_t* vals;
} omap;

static void omap_init(omap* m, int64_t n) {
  int64_t cap = 16;
  while (cap < 2 * n + 16) cap <<= 1;
  m->cap = cap;
  m->keys = (int32_t*)calloc((size_t)cap * 4, sizeof(int32_t));
  m->vals = (int32_t*)calloc((size_t)cap, sizeof(int32_t));
}
static void omap_free(omap* m) {
  free(m->keys);
  free(m->vals);
}
static void sort_small(int32_t* a, int n) {
  for (int i = 1; i < n; i++) {
    int32_t v = a[i];
    int j = i - 1;
    while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; j--; }
    a[j + 1] = v;
  }
}
static uint64_t omap_hash(const int32_t* k) {
  uint64_t h = 0;
  for (int i = 0; i < 4; i++) h = splitmix64(h ^ (uint64_t)(uint32_t)k[i]);
  return h;
}
/* key: n ids (unsorted); returns pointer to value slot, *found set */
static int32_t* omap_slot(omap* m, const int32_t* ids, int n, int* found) {
  int32_t k[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; i++) k[i] = ids[i];
  sort_small(k, n);
  uint64_t h = omap_hash(k) & (uint64_t)(m->cap - 1);
  for (;;) {
    int32_t* s = m->keys + 4 * h;
    if (s[0] == 0) {
      memcpy(s, k, sizeof(k));
      *found = 0;
      return m->vals + h;
    }
    if (s[0] == k[0] && s[1] == k[1] && s[2] == k[2] && s[3] == k[3]) {
      *found = 1;
      return m->vals + h;
    }
    h = (h + 1) & (uint64_t)(m->cap - 1);
  }
}

/* ------------------------------------------------------------------------ */
/* Mesh generation                                                           */
/* ------------------------------------------------------------------------ */

static int64_t prod_i(const int32_t* n, int D) {
  int64_t p = 1;
  for (int d = 0; d < D; d++) p *= n[d];
  return p;
}

/* Sizes of the mesh produced by or_cartesian_mesh.
 * out[0]=nnodes out[1]=ncells out[2]=nodes per cell
 * out[3+d] = number of parent d-faces (boundary faces of the box found by the
 * barrier of src/cartesian_mesh.jl:105-181 / :342-427), d = 0..D-1. */
void or_cartesian_mesh_counts(int D, const int32_t* n, int simplex, int64_t* out) {
  int64_t nn = 1;
  for (int d = 0; d < D; d++) nn *= (n[d] + 1);
  out[0] = nn;
  out[1] = prod_i(n, D) * (simplex ? (D == 3 ? 6 : 2) : 1);
  out[2] = simplex ? D + 1 : (1 << D);
  /* corners */
  out[3] = 1 << D;
  if (D == 2) {
    int64_t e = 2 * (int64_t)n[0] + 2 * (int64_t)n[1];
    out[4] = simplex ? e : e;
  } else if (D == 3) {
    int64_t be = 4 * ((int64_t)n[0] + n[1] + n[2]);
    int64_t bf = 2 * ((int64_t)n[0] * n[1] + (int64_t)n[1] * n[2] + (int64_t)n[0] * n[2]);
    out[4] = be;
    out[5] = simplex ? 2 * bf : bf;
  }
}

/* Reference 6-tet (or 2-triangle) split of the unit cube, complexified:
 * boundary sub-faces of each cube face, in sub-face id order and vertex order
 * of the complexified simplex mesh (src/domain.jl:270-320 -> complexify,
 * src/topology.jl:1594-1704 first-encounter numbering over tets and their
 * local faces, vertex order from the first tet, src/topology.jl:1468-1540).
 * Returns, for each cube face k (0..5), up to 2 triangles (local cube nodes). */
static void cube_face_triangles(int tri[6][2][3], int ntri[6]) {
  /* first-encounter numbering of the triangles of the 6 tets */
  int tverts[24][3];
  int ntris = 0;
  for (int t = 0; t < 6; t++)
    for (int f = 0; f < 4; f++) {
      int v[3];
      for (int i = 0; i < 3; i++) v[i] = CUBE_TETS[t][TET_FACES[f][i] - 1];
      int found = 0;
      for (int s = 0; s < ntris && !found; s++) {
        int m = 0;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) m += (tverts[s][i] == v[j]);
        if (m == 3) found = 1;
      }
      if (!found) {
        memcpy(tverts[ntris], v, sizeof(v));
        ntris++;
      }
    }
  for (int k = 0; k < 6; k++) {
    ntri[k] = 0;
    for (int s = 0; s < ntris; s++) {
      int inface = 1;
      for (int i = 0; i < 3; i++) {
        int ok = 0;
        for (int j = 0; j < 4; j++) ok |= (HEX_FACES[k][j] == tverts[s][i]);
        inface &= ok;
      }
      if (inface) {
        memcpy(tri[k][ntri[k]], tverts[s], sizeof(tverts[s]));
        ntri[k]++;
      }
    }
  }
}

/* Cartesian mesh with boundary faces and groups.
 * cartesian_chain src/cartesian_mesh.jl:213-263 (nodes x-fastest, cell
 * local nodes in CartesianIndices(0:1,...) order); structured_simplex_chain
 * :265-328 (split by src/domain.jl:322-342); boundary barrier :105-181 and
 * :342-427: parent d-faces are the cells' local d-faces whose nodes are all
 * shared by at most 2^d cells, found cell by cell in local-face order; the
 * group of a parent face is its local face index k ("d-face-k").
 * Outputs (1-based node ids):
 *   coords[nnodes*D], cell_nodes[ncells*nv]
 *   pf0[ncorners]                 parent 0-faces (nodes)
 *   pf1[npf1*2], pf1g[npf1]       parent 1-faces (2-D: boundary edges;
 *                                 3-D: box-edge segments) and group k
 *   pf2[npf2*nfv], pf2g[npf2]     3-D only: boundary quads (nfv=4) or
 *                                 triangles (nfv=3, simplex) and group k */
void or_cartesian_mesh(int D, const int32_t* n, const double* box, int simplex,
                       double* coords, int32_t* cell_nodes, int32_t* pf0,
                       int32_t* pf1, int32_t* pf1g, int32_t* pf2, int32_t* pf2g) {
  int32_t np[3] = {1, 1, 1}, nc[3] = {1, 1, 1};
  for (int d = 0; d < D; d++) { np[d] = n[d] + 1; nc[d] = n[d]; }
  int64_t nnodes = (int64_t)np[0] * np[1] * np[2];
  int64_t nhex = (int64_t)nc[0] * nc[1] * nc[2];
  double h[3];
  for (int d = 0; d < D; d++) h[d] = (box[2 * d + 1] - box[2 * d]) / n[d];
  /* node coordinates: pmin + h .* (ci - 1) */
  for (int64_t k = 0; k < nnodes; k++) {
    int64_t r = k;
    for (int d = 0; d < D; d++) {
      int64_t i = r % np[d];
      r /= np[d];
      coords[k * D + d] = box[2 * d] + h[d] * (double)i;
    }
  }
  int nlv = 1 << D;
  int32_t* hexnodes = (int32_t*)malloc(sizeof(int32_t) * nhex * nlv);
  for (int64_t c = 0; c < nhex; c++) {
    int64_t r = c, ci[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) { ci[d] = r % nc[d]; r /= nc[d]; }
    for (int lv = 0; lv < nlv; lv++) {
      int64_t node = 0, stride = 1;
      for (int d = 0; d < D; d++) {
        node += (ci[d] + ((lv >> d) & 1)) * stride;
        stride *= np[d];
      }
      hexnodes[c * nlv + lv] = (int32_t)(node + 1);
    }
  }
  if (!simplex) {
    memcpy(cell_nodes, hexnodes, sizeof(int32_t) * nhex * nlv);
  } else if (D == 3) {
    for (int64_t c = 0; c < nhex; c++)
      for (int t = 0; t < 6; t++)
        for (int i = 0; i < 4; i++)
          cell_nodes[(c * 6 + t) * 4 + i] = hexnodes[c * 8 + CUBE_TETS[t][i] - 1];
  } else {
    static const int SQ_TRIS[2][3] = {{1, 2, 3}, {4, 3, 2}};
    for (int64_t c = 0; c < nhex; c++)
      for (int t = 0; t < 2; t++)
        for (int i = 0; i < 3; i++)
          cell_nodes[(c * 2 + t) * 3 + i] = hexnodes[c * 4 + SQ_TRIS[t][i] - 1];
  }
  /* node_to_n: number of (hex) cells around each node */
  int32_t* cnt = (int32_t*)calloc(nnodes, sizeof(int32_t));
  for (int64_t c = 0; c < nhex; c++)
    for (int lv = 0; lv < nlv; lv++) cnt[hexnodes[c * nlv + lv] - 1]++;
  int tri[6][2][3], ntri[6];
  if (simplex && D == 3) cube_face_triangles(tri, ntri);
  /* d = 0 */
  int64_t k0 = 0, k1 = 0, k2 = 0;
  for (int64_t c = 0; c < nhex; c++)
    for (int lv = 0; lv < nlv; lv++) {
      int32_t node = hexnodes[c * nlv + lv];
      if (cnt[node - 1] <= 1) pf0[k0++] = node;
    }
  /* d = 1 */
  if (D >= 2) {
    int ne = D == 2 ? 4 : 12;
    for (int64_t c = 0; c < nhex; c++)
      for (int le = 0; le < ne; le++) {
        const int* ev = D == 2 ? QUAD_EDGES[le] : HEX_EDGES[le];
        int32_t a = hexnodes[c * nlv + ev[0] - 1], b = hexnodes[c * nlv + ev[1] - 1];
        if (cnt[a - 1] <= 2 && cnt[b - 1] <= 2) {
          pf1[2 * k1] = a;
          pf1[2 * k1 + 1] = b;
          pf1g[k1] = le + 1;
          k1++;
        }
      }
  }
  /* d = 2 (3-D) */
  if (D == 3) {
    for (int64_t c = 0; c < nhex; c++)
      for (int lf = 0; lf < 6; lf++) {
        int bnd = 1;
        for (int i = 0; i < 4; i++)
          if (cnt[hexnodes[c * 8 + HEX_FACES[lf][i] - 1] - 1] > 4) { bnd = 0; break; }
        if (!bnd) continue;
        if (!simplex) {
          for (int i = 0; i < 4; i++) pf2[4 * k2 + i] = hexnodes[c * 8 + HEX_FACES[lf][i] - 1];
          pf2g[k2] = lf + 1;
          k2++;
        } else {
          for (int s = 0; s < ntri[lf]; s++) {
            for (int i = 0; i < 3; i++) pf2[3 * k2 + i] = hexnodes[c * 8 + tri[lf][s][i] - 1];
            pf2g[k2] = lf + 1;
            k2++;
          }
        }
      }
  }
  free(cnt);
  free(hexnodes);
}

/* Jitter interior nodes by U(-amp*h, amp*h) per axis, key = 4*node0+axis. */
void or_jitter_nodes(int D, const int32_t* n, const double* box, double amp, uint64_t seed,
                     double* coords) {
  int64_t np[3] = {1, 1, 1};
  for (int d = 0; d < D; d++) np[d] = n[d] + 1;
  int64_t nnodes = np[0] * np[1] * np[2];
  for (int64_t k = 0; k < nnodes; k++) {
    int64_t r = k, interior = 1;
    for (int d = 0; d < D; d++) {
      int64_t i = r % np[d];
      r /= np[d];
      if (i == 0 || i == np[d] - 1) interior = 0;
    }
    if (!interior) continue;
    for (int d = 0; d < D; d++) {
      double h = (box[2 * d + 1] - box[2 * d]) / n[d];
      double u = or_uniform(seed, 4 * (uint64_t)k + (uint64_t)d);
      coords[k * D + d] += amp * h * (2.0 * u - 1.0);
    }
  }
}

/* Per-cell lognormal(0, sigma) coefficient from Box-Muller of two keyed
 * uniforms (keys 2*cell0 and 2*cell0+1 under seed ^ 0xC0EFF1C1E47). */
void or_lognormal_cells(int64_t ncells, double sigma, uint64_t seed, double* out) {
  uint64_t s = seed ^ 0xC0EFF1C1E47ULL;
  for (int64_t c = 0; c < ncells; c++) {
    double u1 = or_uniform(s, 2 * (uint64_t)c), u2 = or_uniform(s, 2 * (uint64_t)c + 1);
    double z = sqrt(-2.0 * log(1.0 - u1)) * cos(6.283185307179586 * u2);
    out[c] = exp(sigma * z);
  }
}

/* ------------------------------------------------------------------------ */
/* Topology numbering                                                        */
/* ------------------------------------------------------------------------ */

/* create_vertices! src/topology.jl:1034-1097 for a linear mesh (every node is
 * a vertex): nodes of existing parent 0-faces get ids first in parent order,
 * the rest follow in node order.  node_vertex[nnodes] (1-based). */
int64_t or_vertex_ids(int64_t nnodes, int64_t npf0, const int32_t* pf0, int32_t* node_vertex) {
  for (int64_t k = 0; k < nnodes; k++) node_vertex[k] = -1;
  int32_t v = 0;
  for (int64_t i = 0; i < npf0; i++) {
    int32_t node = pf0[i];
    if (node_vertex[node - 1] == -1) node_vertex[node - 1] = ++v;
  }
  for (int64_t k = 0; k < nnodes; k++)
    if (node_vertex[k] == -1) node_vertex[k] = ++v;
  return v;
}

/* generate_face_boundary src/topology.jl:1594-1704 with generate_face_vertices
 * :1468-1540.  Creates the d-faces of a set of n-faces (d = n-1): existing
 * parent d-faces keep ids 1..npar; others get new ids in the order in which
 * the scan over n-faces (and their local d-faces) meets them.  A new d-face
 * takes its vertex order from the first n-face that meets it.
 *   nf_verts[nn*nlv]: vertex ids of each n-face
 *   ldf[nld][ndv]:    local d-face -> local vertices (1-based), flattened
 *   par[npar*ndv]:    parent d-face vertex ids
 * outputs nf_dfaces[nn*nld] (1-based) and df_verts[(cap)*ndv]; returns count. */
int64_t or_face_boundary(int64_t nn, int nlv, const int32_t* nf_verts, int nld, int ndv,
                         const int32_t* ldf, int64_t npar, const int32_t* par,
                         int32_t* nf_dfaces, int32_t* df_verts) {
  omap m;
  omap_init(&m, npar + nn * nld);
  int found;
  for (int64_t p = 0; p < npar; p++) {
    int32_t* s = omap_slot(&m, par + p * ndv, ndv, &found);
    *s = (int32_t)(p + 1);
    memcpy(df_verts + p * ndv, par + p * ndv, sizeof(int32_t) * ndv);
  }
  int64_t next = npar;
  int32_t v[4];
  for (int64_t f = 0; f < nn; f++)
    for (int l = 0; l < nld; l++) {
      for (int i = 0; i < ndv; i++) v[i] = nf_verts[f * nlv + ldf[l * ndv + i] - 1];
      int32_t* s = omap_slot(&m, v, ndv, &found);
      if (!found) {
        *s = (int32_t)(++next);
        memcpy(df_verts + (next - 1) * ndv, v, sizeof(int32_t) * ndv);
      }
      nf_dfaces[f * nld + l] = *s;
    }
  omap_free(&m);
  return next;
}

/* fill_face_boundary_mesh_topology! src/topology.jl:515-591: local d-faces of
 * each cell looked up (by vertex set) among existing d-faces. */
void or_face_lookup(int64_t nc, int nlv, const int32_t* c_verts, int nld, int ndv,
                    const int32_t* ldf, int64_t ndf, const int32_t* df_verts, int32_t* c_dfaces) {
  omap m;
  omap_init(&m, ndf);
  int found;
  for (int64_t p = 0; p < ndf; p++) *omap_slot(&m, df_verts + p * ndv, ndv, &found) = (int32_t)(p + 1);
  int32_t v[4];
  for (int64_t c = 0; c < nc; c++)
    for (int l = 0; l < nld; l++) {
      for (int i = 0; i < ndv; i++) v[i] = c_verts[c * nlv + ldf[l * ndv + i] - 1];
      int32_t* s = omap_slot(&m, v, ndv, &found);
      c_dfaces[c * nld + l] = found ? *s : 0;
    }
  omap_free(&m);
}

/* ------------------------------------------------------------------------ */
/* Lagrange reference elements (src/space.jl:1127-1177, :1257-1286)          */
/* ------------------------------------------------------------------------ */

/* Number of local nodes of the space on a cell type. */
static int space_nodes(int ctype, int order) {
  if (ctype == OR_TET4) return order == 2 ? 10 : 4;
  int D = ctype == OR_QUAD4 ? 2 : 3;
  int m = order + 1;
  return D == 2 ? m * m : m * m * m;
}

/* Q_k node index (0-based) from exponents (first index fastest). */
static int qnode(int D, int order, const int* e) {
  int m = order + 1;
  return D == 2 ? e[0] + m * e[1] : e[0] + m * (e[1] + m * e[2]);
}

/* Q_k nodes of the closure of the local (D-1)-face lf; returns count. */
/* P2 tetrahedron: nodes are the exponents (a,b,c), a+b+c <= 2, first index
 * fastest (src/space.jl:1127-1146 with space_type :P): vertices at nodes
 * 0, 2, 5, 9, midpoints of the local edges 12 13 23 14 24 34 at 1 3 4 6 7 8 */
static const int P2_VERT[4] = {0, 2, 5, 9};
static const int P2_EDGE[6] = {1, 3, 4, 6, 7, 8};
static const int TET_EDGES[6][2] = {{1, 2}, {1, 3}, {2, 3}, {1, 4}, {2, 4}, {3, 4}};

static int face_closure_nodes(int ctype, int order, int lf, int* out) {
  if (ctype == OR_TET4 && order == 2) {
    int cnt = 0;
    for (int i = 0; i < 3; i++) out[cnt++] = P2_VERT[TET_FACES[lf][i] - 1];
    for (int e = 0; e < 6; e++) {
      int in = 0;
      for (int i = 0; i < 3; i++) in += (TET_EDGES[e][0] == TET_FACES[lf][i]) + (TET_EDGES[e][1] == TET_FACES[lf][i]);
      if (in == 2) out[cnt++] = P2_EDGE[e];
    }
    return cnt;
  }
  if (ctype == OR_TET4) {
    for (int i = 0; i < 3; i++) out[i] = TET_FACES[lf][i] - 1;
    return 3;
  }
  int D = ctype == OR_QUAD4 ? 2 : 3, m = order + 1, cnt = 0;
  /* face lf fixes one direction at 0 or 1: quad edges 1..4 = y0,y1,x0,x1;
   * hex faces 1..6 = z0,z1,y0,y1,x0,x1 */
  int dir, side;
  if (D == 2) { dir = lf < 2 ? 1 : 0; side = lf & 1; }
  else { dir = 2 - lf / 2; side = lf & 1; }
  int nn = space_nodes(ctype, order);
  for (int k = 0; k < nn; k++) {
    int e[3] = {k % m, (k / m) % m, k / (m * m)};
    if (e[dir] == side * order) out[cnt++] = k;
  }
  return cnt;
}

/* 1-D Lagrange basis on equispaced nodes of order 1 or 2. */
static void lag1d(int order, double x, double* v, double* dv) {
  if (order == 1) {
    v[0] = 1.0 - x; v[1] = x;
    dv[0] = -1.0; dv[1] = 1.0;
  } else {
    v[0] = 2.0 * (x - 0.5) * (x - 1.0);
    v[1] = -4.0 * x * (x - 1.0);
    v[2] = 2.0 * x * (x - 0.5);
    dv[0] = 4.0 * x - 3.0;
    dv[1] = -8.0 * x + 4.0;
    dv[2] = 4.0 * x - 1.0;
  }
}

/* Shape values/gradients of a reference space at a point. */
static void tabulate(int ctype, int order, const double* x, double* val, double* grad) {
  if (ctype == OR_TET4 && order == 2) {
    /* P2 Lagrange basis in barycentric form: l_i (2 l_i - 1) at vertex i,
     * 4 l_i l_j at the midpoint of edge ij */
    double l[4] = {1.0 - x[0] - x[1] - x[2], x[0], x[1], x[2]};
    double gl[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 4; i++) {
      int n = P2_VERT[i];
      val[n] = l[i] * (2.0 * l[i] - 1.0);
      for (int d = 0; d < 3; d++) grad[n * 3 + d] = (4.0 * l[i] - 1.0) * gl[i][d];
    }
    for (int e = 0; e < 6; e++) {
      int i = TET_EDGES[e][0] - 1, j = TET_EDGES[e][1] - 1, n = P2_EDGE[e];
      val[n] = 4.0 * l[i] * l[j];
      for (int d = 0; d < 3; d++) grad[n * 3 + d] = 4.0 * (l[j] * gl[i][d] + l[i] * gl[j][d]);
    }
    return;
  }
  if (ctype == OR_TET4) {
    val[0] = 1.0 - x[0] - x[1] - x[2];
    val[1] = x[0]; val[2] = x[1]; val[3] = x[2];
    double g[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    memcpy(grad, g, sizeof(g));
    return;
  }
  int D = ctype == OR_QUAD4 ? 2 : 3, m = order + 1;
  double v[3][3], dv[3][3];
  for (int d = 0; d < D; d++) lag1d(order, x[d], v[d], dv[d]);
  int nn = space_nodes(ctype, order);
  for (int k = 0; k < nn; k++) {
    int e[3] = {k % m, (k / m) % m, k / (m * m)};
    double p = 1.0;
    for (int d = 0; d < D; d++) p *= v[d][e[d]];
    val[k] = p;
    for (int d = 0; d < D; d++) {
      double g = 1.0;
      for (int d2 = 0; d2 < D; d2++) g *= (d2 == d) ? dv[d2][e[d2]] : v[d2][e[d2]];
      grad[k * D + d] = g;
    }
  }
}

/* Quadrature: tensor Gauss-Legendre with ceil((deg+1)/2) points per
 * direction, first index fastest (src/quadrature.jl:78-106), or the 4-point
 * Strang rule on the tetrahedron (src/quadrature.jl:512-529).  Returns npts. */
int or_quadrature(int ctype, int degree, double* x, double* w) {
  if (ctype == OR_TET4 && degree > 2) {
    /* degrees 3-4: the reference's strang_quadrature_4 (src/quadrature.jl:
     * 554-590), Keast's 11-point rule: centroid, (11/14, 1/14, 1/14) and
     * permutations with (1/14, 1/14, 1/14), the 6 points with coordinates
     * (1 +- sqrt(5/14))/4 */
    if (degree > 4) return -1;
    double r = sqrt(5.0 / 14.0), a = 0.25 * (1.0 + r), b = 0.25 * (1.0 - r), f = 11.0 / 14.0, g = 1.0 / 14.0;
    double p[11][3] = {{0.25, 0.25, 0.25}, {f, g, g}, {g, f, g}, {g, g, f}, {g, g, g}, {a, a, b},
                       {a, b, a}, {a, b, b}, {b, a, a}, {b, a, b}, {b, b, a}};
    for (int q = 0; q < 11; q++) {
      for (int d = 0; d < 3; d++) x[3 * q + d] = p[q][d];
      w[q] = q == 0 ? -74.0 / 5625.0 : (q < 5 ? 343.0 / 45000.0 : 56.0 / 2250.0);
    }
    return 11;
  }
  if (ctype == OR_TET4) {
    double a = 0.5854101966249685, b = 0.1381966011250105, c = 1.0 / 24.0;
    double p[4][3] = {{b, b, b}, {a, b, b}, {b, a, b}, {b, b, a}};
    for (int q = 0; q < 4; q++) {
      for (int d = 0; d < 3; d++) x[3 * q + d] = p[q][d];
      w[q] = c;
    }
    return 4;
  }
  int D = ctype == OR_QUAD4 ? 2 : 3;
  int n1 = (degree + 2) / 2;
  double g[3], gw[3];
  if (n1 == 1) { g[0] = 0.5; gw[0] = 1.0; }
  else if (n1 == 2) {
    double s = 0.5 / sqrt(3.0);
    g[0] = 0.5 - s; g[1] = 0.5 + s; gw[0] = gw[1] = 0.5;
  } else if (n1 == 3) {
    double s = 0.5 * sqrt(0.6);
    g[0] = 0.5 - s; g[1] = 0.5; g[2] = 0.5 + s;
    gw[0] = 5.0 / 18.0; gw[1] = 8.0 / 18.0; gw[2] = 5.0 / 18.0;
  } else return -1;
  int nq = D == 2 ? n1 * n1 : n1 * n1 * n1;
  for (int q = 0; q < nq; q++) {
    int i[3] = {q % n1, (q / n1) % n1, q / (n1 * n1)};
    double ww = 1.0;
    for (int d = 0; d < D; d++) { x[D * q + d] = g[i[d]]; ww *= gw[i[d]]; }
    w[q] = ww;
  }
  return nq;
}

/* ------------------------------------------------------------------------ */
/* DOF numbering: generate_dof_ids step_1 / step_2                           */
/* ------------------------------------------------------------------------ */

/* Local Q_k node of a local vertex (0-based) of the cube. */
static int vertex_qnode(int D, int order, int lv) {
  int e[3] = {0, 0, 0};
  for (int d = 0; d < D; d++) e[d] = ((lv >> d) & 1) * order;
  return qnode(D, order, e);
}
/* Q2 node at the centroid of local vertices */
static int centroid_qnode(int D, const int* lvs, int nv) {
  int e[3] = {0, 0, 0};
  for (int i = 0; i < nv; i++)
    for (int d = 0; d < D; d++) e[d] += ((lvs[i] - 1) >> d) & 1;
  for (int d = 0; d < D; d++) e[d] = (2 * e[d]) / nv;
  return qnode(D, 2, e);
}

/* generate_dof_ids_step_1 src/space.jl:327-466 (offsets per d-face, vertex
 * -> edge -> face -> cell, dof = offset + own index; component-major local
 * numbering ldof = node*ncomp + comp, src/space.jl:1257-1286) followed by
 * generate_dof_ids_step_2 :477-535 (dofs in the closure of tagged (D-1)-faces
 * are Dirichlet; free dofs first in stable order, partition_from_mask
 * :910-920; Dirichlet ids negative).
 *   c_verts[nc*nlv]     vertex ids of each cell
 *   c_edges[nc*nle]     edge ids (Q2 only, else NULL)
 *   c_faces[nc*6]       3-D face ids (Q2 hex only, else NULL)
 *   c_tagged[nc*nlf]    1 if local (D-1)-face is a tagged Dirichlet face
 * outputs cell_dofs[nc*nloc], returns nfree (ndiri in *ndiri). */
int64_t or_dof_ids(int ctype, int order, int ncomp, int64_t nc, const int32_t* c_verts,
                   int64_t nverts, const int32_t* c_edges, int64_t nedges,
                   const int32_t* c_faces, int64_t nfaces, const uint8_t* c_tagged,
                   int32_t* cell_dofs, int64_t* ndiri) {
  int D = ctype == OR_QUAD4 ? 2 : 3;
  int nlv = ctype == OR_TET4 ? 4 : (1 << D);
  int nn = space_nodes(ctype, order);
  int nloc = nn * ncomp;
  int nlf = ctype == OR_TET4 ? 4 : 2 * D;
  int nle = D == 2 ? 4 : 12;
  /* P2 tets own dofs on vertices and edges only */
  const int tet2 = ctype == OR_TET4 && order == 2;
  int64_t off_e = nverts * ncomp;
  int64_t off_f = off_e + (order == 2 ? nedges * ncomp : 0);
  int64_t off_c = off_f + ((order == 2 && D == 3 && !tet2) ? nfaces * ncomp : 0);
  int64_t ndofs = off_c + (order == 2 && !tet2 ? nc * ncomp : 0);
  for (int64_t c = 0; c < nc; c++) {
    int32_t* cd = cell_dofs + c * nloc;
    for (int lv = 0; lv < nlv; lv++) {
      int node = tet2 ? P2_VERT[lv] : ((ctype == OR_TET4 || order == 1) ? lv : vertex_qnode(D, order, lv));
      int64_t v = c_verts[c * nlv + lv];
      for (int k = 0; k < ncomp; k++) cd[node * ncomp + k] = (int32_t)((v - 1) * ncomp + k + 1);
    }
    if (tet2) {
      for (int le = 0; le < 6; le++) {
        int64_t e = c_edges[c * 6 + le];
        for (int k = 0; k < ncomp; k++)
          cd[P2_EDGE[le] * ncomp + k] = (int32_t)(off_e + (e - 1) * ncomp + k + 1);
      }
    } else if (order == 2) {
      for (int le = 0; le < nle; le++) {
        const int* ev = D == 2 ? QUAD_EDGES[le] : HEX_EDGES[le];
        int node = centroid_qnode(D, ev, 2);
        int64_t e = c_edges[c * nle + le];
        for (int k = 0; k < ncomp; k++)
          cd[node * ncomp + k] = (int32_t)(off_e + (e - 1) * ncomp + k + 1);
      }
      if (D == 3)
        for (int lf = 0; lf < 6; lf++) {
          int node = centroid_qnode(3, HEX_FACES[lf], 4);
          int64_t f = c_faces[c * 6 + lf];
          for (int k = 0; k < ncomp; k++)
            cd[node * ncomp + k] = (int32_t)(off_f + (f - 1) * ncomp + k + 1);
        }
      int node = D == 2 ? 4 : 13;
      for (int k = 0; k < ncomp; k++) cd[node * ncomp + k] = (int32_t)(off_c + c * ncomp + k + 1);
    }
  }
  /* step 2 */
  uint8_t* tag = (uint8_t*)calloc(ndofs, 1);
  int fn[16];
  for (int64_t c = 0; c < nc; c++)
    for (int lf = 0; lf < nlf; lf++) {
      if (!c_tagged[c * nlf + lf]) continue;
      int cnt = face_closure_nodes(ctype, order, lf, fn);
      for (int i = 0; i < cnt; i++)
        for (int k = 0; k < ncomp; k++) tag[cell_dofs[c * nloc + fn[i] * ncomp + k] - 1] = 1;
    }
  int32_t* perm = (int32_t*)malloc(sizeof(int32_t) * ndofs);
  int64_t nfree = 0, nd = 0;
  for (int64_t i = 0; i < ndofs; i++)
    if (!tag[i]) perm[i] = (int32_t)(++nfree);
  for (int64_t i = 0; i < ndofs; i++)
    if (tag[i]) perm[i] = (int32_t)(-(++nd));
  for (int64_t i = 0; i < nc * nloc; i++) cell_dofs[i] = perm[cell_dofs[i] - 1];
  free(perm);
  free(tag);
  *ndiri = nd;
  return nfree;
}

/* Tags of the cells' local (D-1)-faces: a local face is tagged when its
 * vertex set is one of the given tagged faces (src/space.jl:487-508 tags by
 * face id; the ids of the tagged faces are those of the named groups). */
void or_tag_cell_faces(int ctype, int64_t nc, const int32_t* c_verts, int64_t nt,
                       const int32_t* t_verts, uint8_t* c_tagged) {
  int D = ctype == OR_QUAD4 ? 2 : 3;
  int nlv = ctype == OR_TET4 ? 4 : (1 << D);
  int nlf = ctype == OR_TET4 ? 4 : 2 * D;
  int ndv = ctype == OR_TET4 ? 3 : (D == 2 ? 2 : 4);
  omap m;
  omap_init(&m, nt);
  int found;
  for (int64_t t = 0; t < nt; t++) *omap_slot(&m, t_verts + t * ndv, ndv, &found) = 1;
  int32_t v[4];
  for (int64_t c = 0; c < nc; c++)
    for (int lf = 0; lf < nlf; lf++) {
      for (int i = 0; i < ndv; i++) {
        int lv = ctype == OR_TET4 ? TET_FACES[lf][i] : (D == 2 ? QUAD_EDGES[lf][i] : HEX_FACES[lf][i]);
        v[i] = c_verts[c * nlv + lv - 1];
      }
      /* lookup without insertion */
      int32_t k[4] = {0, 0, 0, 0};
      for (int i = 0; i < ndv; i++) k[i] = v[i];
      sort_small(k, ndv);
      uint64_t h = omap_hash(k) & (uint64_t)(m.cap - 1);
      int hit = 0;
      for (;;) {
        int32_t* s = m.keys + 4 * h;
        if (s[0] == 0) break;
        if (s[0] == k[0] && s[1] == k[1] && s[2] == k[2] && s[3] == k[3]) { hit = 1; break; }
        h = (h + 1) & (uint64_t)(m.cap - 1);
      }
      c_tagged[c * nlf + lf] = (uint8_t)hit;
    }
  omap_free(&m);
}

/* ------------------------------------------------------------------------ */
/* Per-cell integration (the generated loop, src/compiler.jl:1865-1917)      */
/* ------------------------------------------------------------------------ */

typedef struct {
  int ctype, order, ncomp, D, nlv, nn, nloc, nq;
  double qx[27 * 3], qw[27];
  double gval[27][8], ggrad[27][8 * 3];       /* geometry map (P1/Q1) */
  double sval[27][27], sgrad[27][27 * 3];     /* space */
} elem_t;

static void elem_init(elem_t* e, int ctype, int order, int ncomp, int degree) {
  e->ctype = ctype; e->order = order; e->ncomp = ncomp;
  e->D = ctype == OR_QUAD4 ? 2 : 3;
  e->nlv = ctype == OR_TET4 ? 4 : (1 << e->D);
  e->nn = space_nodes(ctype, order);
  e->nloc = e->nn * ncomp;
  e->nq = or_quadrature(ctype, degree, e->qx, e->qw);
  for (int q = 0; q < e->nq; q++) {
    tabulate(ctype, 1, e->qx + e->D * q, e->gval[q], e->ggrad[q]);
    tabulate(ctype, order, e->qx + e->D * q, e->sval[q], e->sgrad[q]);
  }
}

/* Jacobian J = sum_n x_n (x) grad m_n (src/accessors.jl:941-968), its
 * inverse and determinant. */
static double jac(const elem_t* e, int q, const double* X, double* invJ) {
  int D = e->D;
  double J[9] = {0};
  for (int n = 0; n < e->nlv; n++)
    for (int i = 0; i < D; i++)
      for (int j = 0; j < D; j++) J[i * D + j] += X[n * D + i] * e->ggrad[q][n * D + j];
  double det;
  if (D == 2) {
    det = J[0] * J[3] - J[1] * J[2];
    invJ[0] = J[3] / det; invJ[1] = -J[1] / det;
    invJ[2] = -J[2] / det; invJ[3] = J[0] / det;
  } else {
    double c00 = J[4] * J[8] - J[5] * J[7], c01 = J[5] * J[6] - J[3] * J[8], c02 = J[3] * J[7] - J[4] * J[6];
    det = J[0] * c00 + J[1] * c01 + J[2] * c02;
    invJ[0] = c00 / det; invJ[3] = c01 / det; invJ[6] = c02 / det;
    invJ[1] = (J[2] * J[7] - J[1] * J[8]) / det;
    invJ[4] = (J[0] * J[8] - J[2] * J[6]) / det;
    invJ[7] = (J[1] * J[6] - J[0] * J[7]) / det;
    invJ[2] = (J[1] * J[5] - J[2] * J[4]) / det;
    invJ[5] = (J[2] * J[3] - J[0] * J[5]) / det;
    invJ[8] = (J[0] * J[4] - J[1] * J[3]) / det;
  }
  return det;
}

/* Element matrix Ke[i*nloc+j] (i test, j trial) of one cell.
 * Laplacian: coef * grad(u).grad(v) (docs example_poisson_equation.jl:77);
 * mass: coef * u v (test/problems_tests.jl:53);
 * elasticity: sigma(eps(u)):eps(v), sigma = lam tr(eps) I + 2 mu eps,
 * lam = E nu/((1+nu)(1-2nu)), mu = E/(2(1+nu)) with E = coef
 * (docs example_linear_elasticity.jl:76-111); grad phi = J^-T grad_ref phi
 * (src/accessors.jl:1365-1368); dV = |det J| w (src/quadrature.jl:4-6). */
static void elem_matrix(const elem_t* e, int form, double coef, double nu, const double* X, double* Ke) {
  int D = e->D, nn = e->nn, nc = e->ncomp, nloc = e->nloc;
  memset(Ke, 0, sizeof(double) * nloc * nloc);
  double g[27 * 3];
  double lam = coef * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), mu = coef / (2.0 * (1.0 + nu));
  for (int q = 0; q < e->nq; q++) {
    double invJ[9];
    double det = jac(e, q, X, invJ);
    double dV = fabs(det) * e->qw[q];
    for (int n = 0; n < nn; n++)
      for (int d = 0; d < D; d++) {
        double s = 0.0;
        for (int k = 0; k < D; k++) s += invJ[k * D + d] * e->sgrad[q][n * D + k];
        g[n * D + d] = s;
      }
    for (int j = 0; j < nloc; j++) {
      int m = j / nc, dj = j % nc;
      for (int i = 0; i < nloc; i++) {
        int n = i / nc, ci = i % nc;
        double v;
        if (form == OR_LAPLACE) {
          if (ci != dj) continue;
          double dot = 0.0;
          for (int d = 0; d < D; d++) dot += g[m * D + d] * g[n * D + d];
          v = coef * dot;
        } else if (form == OR_MASS) {
          if (ci != dj) continue;
          v = coef * (e->sval[q][m] * e->sval[q][n]);
        } else {
          /* grad u = e_dj (x) g_m ; grad v = e_ci (x) g_n */
          double eu[9] = {0}, ev[9] = {0}, su[9];
          for (int a = 0; a < D; a++)
            for (int b = 0; b < D; b++) {
              double gu = (a == dj) ? g[m * D + b] : 0.0, gut = (b == dj) ? g[m * D + a] : 0.0;
              double gv = (a == ci) ? g[n * D + b] : 0.0, gvt = (b == ci) ? g[n * D + a] : 0.0;
              eu[a * D + b] = 0.5 * (gu + gut);
              ev[a * D + b] = 0.5 * (gv + gvt);
            }
          double tr = 0.0;
          for (int a = 0; a < D; a++) tr += eu[a * D + a];
          for (int a = 0; a < D; a++)
            for (int b = 0; b < D; b++) su[a * D + b] = lam * tr * (a == b) + 2.0 * mu * eu[a * D + b];
          v = 0.0;
          for (int a = 0; a < D * D; a++) v += su[a] * ev[a];
        }
        Ke[i * nloc + j] += v * dV;
      }
    }
  }
}

/* Element vector of int f v dOmega with a constant (vector) source f. */
static void elem_vector(const elem_t* e, const double* f, double coef, const double* X, double* be) {
  int nn = e->nn, nc = e->ncomp;
  memset(be, 0, sizeof(double) * e->nloc);
  for (int q = 0; q < e->nq; q++) {
    double invJ[9];
    double dV = fabs(jac(e, q, X, invJ)) * e->qw[q];
    for (int n = 0; n < nn; n++)
      for (int k = 0; k < nc; k++) be[n * nc + k] += (coef * f[k] * e->sval[q][n]) * dV;
  }
}

static void gather_x(const elem_t* e, const int32_t* cn, const double* coords, double* X) {
  for (int n = 0; n < e->nlv; n++)
    for (int d = 0; d < e->D; d++) X[n * e->D + d] = coords[(int64_t)(cn[n] - 1) * e->D + d];
}

/* ------------------------------------------------------------------------ */
/* Matrix assembly: counting pass, COO append, COO -> CSC                    */
/* ------------------------------------------------------------------------ */

/* Counting pass (allocate_matrix_barrier_impl! src/assembly.jl:119-153):
 * number of contributions of every cell with free rows and free columns
 * (coldiri = 0) or Dirichlet columns (coldiri = 1, the FREE x DIRICHLET
 * block of src/problems.jl:363-380); cell_off[nc+1]. */
int64_t or_count_coo(int64_t nc, int nloc, const int32_t* cell_dofs, int coldiri, int64_t* cell_off) {
  cell_off[0] = 0;
  for (int64_t c = 0; c < nc; c++) {
    int64_t f = 0, g = 0;
    for (int i = 0; i < nloc; i++) {
      f += cell_dofs[c * nloc + i] > 0;
      g += cell_dofs[c * nloc + i] < 0;
    }
    cell_off[c + 1] = cell_off[c] + f * (coldiri ? g : f);
  }
  return cell_off[nc];
}

/* Integration + contribute! (src/assembly.jl:189-208 with skip_dof :155-157
 * and the COO append :545-556): per cell, j (trial) outer, i (test) inner,
 * skipping Dirichlet dofs.  I, J 0-based rows/cols. */
void or_fill_coo(int ctype, int order, int ncomp, int degree, int form, double nu,
                 int64_t nc, const int32_t* cell_nodes, const double* coords,
                 const int32_t* cell_dofs, const double* coef, int coldiri,
                 const int64_t* cell_off, int32_t* I, int32_t* J, double* V) {
  elem_t e;
  elem_init(&e, ctype, order, ncomp, degree);
  int nloc = e.nloc;
#pragma omp parallel
  {
    double* Ke = (double*)malloc(sizeof(double) * nloc * nloc);
    double X[8 * 3];
#pragma omp for schedule(static)
    for (int64_t c = 0; c < nc; c++) {
      gather_x(&e, cell_nodes + c * e.nlv, coords, X);
      elem_matrix(&e, form, coef ? coef[c] : 1.0, nu, X, Ke);
      const int32_t* cd = cell_dofs + c * nloc;
      int64_t p = cell_off[c];
      for (int j = 0; j < nloc; j++) {
        if (coldiri ? cd[j] > 0 : cd[j] < 0) continue;
        for (int i = 0; i < nloc; i++) {
          if (cd[i] < 0) continue;
          I[p] = cd[i] - 1;
          J[p] = coldiri ? -cd[j] - 1 : cd[j] - 1;
          V[p] = Ke[i * nloc + j];
          p++;
        }
      }
    }
    free(Ke);
  }
}

static int cmp_pair(const void* a, const void* b) {
  const int64_t* x = (const int64_t*)a;
  const int64_t* y = (const int64_t*)b;
  if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
  return x[1] < y[1] ? -1 : (x[1] > y[1]);
}

/* compress -> PartitionedArrays.sparse_matrix (src/assembly.jl:571-575):
 * COO -> CSC with row indices sorted in each column and duplicates summed
 * in COO order.  Counting sort by column (stable), then a stable sort by
 * row inside each column.  colptr[ncols+1], rowval/nzval sized n (worst).
 * Returns nnz. */
int64_t or_coo_to_csc(int64_t n, const int32_t* I, const int32_t* J, const double* V,
                      int64_t ncols, int64_t* colptr, int32_t* rowval, double* nzval) {
  int64_t* cnt = (int64_t*)calloc(ncols + 1, sizeof(int64_t));
  for (int64_t k = 0; k < n; k++) cnt[J[k] + 1]++;
  for (int64_t c = 0; c < ncols; c++) cnt[c + 1] += cnt[c];
  int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * (ncols + 1));
  memcpy(pos, cnt, sizeof(int64_t) * (ncols + 1));
  int64_t* perm = (int64_t*)malloc(sizeof(int64_t) * n);
  for (int64_t k = 0; k < n; k++) perm[pos[J[k]]++] = k;
  free(pos);
  int64_t* nnz_col = (int64_t*)calloc(ncols, sizeof(int64_t));
#pragma omp parallel
  {
    int64_t cap = 0;
    int64_t* tmp = NULL;
#pragma omp for schedule(dynamic, 256)
    for (int64_t c = 0; c < ncols; c++) {
      int64_t b = cnt[c], e = cnt[c + 1], m = e - b;
      if (m > cap) { cap = 2 * m; tmp = (int64_t*)realloc(tmp, sizeof(int64_t) * 2 * cap); }
      for (int64_t k = 0; k < m; k++) { tmp[2 * k] = I[perm[b + k]]; tmp[2 * k + 1] = perm[b + k]; }
      qsort(tmp, (size_t)m, 2 * sizeof(int64_t), cmp_pair); /* (row, coo index): stable */
      int64_t w = b;
      for (int64_t k = 0; k < m; k++) {
        if (k > 0 && tmp[2 * k] == tmp[2 * (k - 1)]) {
          nzval[w - 1] += V[tmp[2 * k + 1]];
        } else {
          rowval[w] = (int32_t)tmp[2 * k];
          nzval[w] = V[tmp[2 * k + 1]];
          w++;
        }
      }
      nnz_col[c] = w - b;
    }
    free(tmp);
  }
  /* compact */
  int64_t w = 0;
  colptr[0] = 0;
  for (int64_t c = 0; c < ncols; c++) {
    int64_t b = cnt[c];
    if (w != b) {
      memmove(rowval + w, rowval + b, sizeof(int32_t) * nnz_col[c]);
      memmove(nzval + w, nzval + b, sizeof(double) * nnz_col[c]);
    }
    w += nnz_col[c];
    colptr[c + 1] = w;
  }
  free(nnz_col);
  free(perm);
  free(cnt);
  return w;
}

/* assemble_vector: allocate_vector + contribute! + dense_vector
 * (src/assembly.jl:27-73, :558-569); free dofs only. */
void or_assemble_vector(int ctype, int order, int ncomp, int degree, const double* f,
                        int64_t nc, const int32_t* cell_nodes, const double* coords,
                        const int32_t* cell_dofs, const double* coef, int64_t nfree, double* b) {
  elem_t e;
  elem_init(&e, ctype, order, ncomp, degree);
  double be[81], X[24];
  memset(b, 0, sizeof(double) * nfree);
  for (int64_t c = 0; c < nc; c++) {
    gather_x(&e, cell_nodes + c * e.nlv, coords, X);
    elem_vector(&e, f, coef ? coef[c] : 1.0, X, be);
    for (int i = 0; i < e.nloc; i++) {
      int32_t d = cell_dofs[c * e.nloc + i];
      if (d > 0) b[d - 1] += be[i];
    }
  }
}

/* Neumann term int g . v dGamma over tagged boundary faces, the loop of
 * assemble_in_Γn! (docs/src/src_jl/example_poisson_equation.jl:161-203)
 * with a constant g (ncomp values):
 *  - faces are visited in the order of the tagged-face list (the faces of
 *    the boundary domain); each one is found among the cells' local faces by
 *    its vertex set (fill_face_boundary_mesh_topology!, src/topology.jl:
 *    515-591), which gives its cell c and local face lf;
 *  - the face's reference quadrature of the given degree: tensor
 *    Gauss-Legendre on a segment or square (src/quadrature.jl:78-106); on a
 *    triangle the reference uses the collapsed (Duffy) rule of
 *    src/quadrature.jl:121-153 -- restated here as Gauss-Legendre in both
 *    collapsed coordinates with the collapse factor (1 - u) in the weight,
 *    exact like the reference's rule for the polynomial integrands of this
 *    term (degree <= order on a flat face), so the two agree to rounding;
 *  - the face point mapped into the cell's reference coordinates, the cell's
 *    shape values there, dGamma = sqrt(det(T^T T)) w with T the tangents
 *    J dxi/ds of the geometry map (change_of_measure, src/quadrature.jl:4-6);
 *  - contribute! of the face-closure DOFs, skipping Dirichlet DOFs
 *    (src/assembly.jl:27-73): b[dof] += be in face order.
 * t_verts: nt tagged faces as vertex ids (ndv each); c_verts: cells' vertex
 * ids.  b (nfree) is accumulated into. */
void or_assemble_boundary_vector(int ctype, int order, int ncomp, int degree, const double* g, int64_t nc,
                                 const int32_t* cell_nodes, const double* coords, const int32_t* cell_dofs,
                                 const int32_t* c_verts, int64_t nt, const int32_t* t_verts, double* b) {
  const int D = ctype == OR_QUAD4 ? 2 : 3;
  const int nlv = ctype == OR_TET4 ? 4 : (1 << D);
  const int nlf = ctype == OR_TET4 ? 4 : 2 * D;
  const int ndv = ctype == OR_TET4 ? 3 : (D == 2 ? 2 : 4);
  const int nn = space_nodes(ctype, order), nloc = nn * ncomp;
  /* reference coordinates of the cell's vertices */
  double xv[8][3];
  for (int v = 0; v < nlv; v++)
    for (int d = 0; d < 3; d++)
      xv[v][d] = ctype == OR_TET4 ? (v == d + 1 ? 1.0 : 0.0) : (d < D ? (double)((v >> d) & 1) : 0.0);
  /* 1-D Gauss-Legendre on [0,1] with n points (n = 1..4) */
  double gp[4], gw[4];
  int n1 = (degree + 2) / 2;
  if (ctype == OR_TET4) n1 = n1 + 1; /* one more point for the (1 - u) factor */
  if (n1 > 4) n1 = 4;
  if (n1 == 1) { gp[0] = 0.5; gw[0] = 1.0; }
  else if (n1 == 2) { double s = 0.5 / sqrt(3.0); gp[0] = 0.5 - s; gp[1] = 0.5 + s; gw[0] = gw[1] = 0.5; }
  else if (n1 == 3) {
    double s = 0.5 * sqrt(0.6);
    gp[0] = 0.5 - s; gp[1] = 0.5; gp[2] = 0.5 + s;
    gw[0] = gw[2] = 5.0 / 18.0; gw[1] = 8.0 / 18.0;
  } else {
    double a = sqrt(3.0 / 7.0 - 2.0 / 7.0 * sqrt(1.2)), c = sqrt(3.0 / 7.0 + 2.0 / 7.0 * sqrt(1.2));
    double wa = (18.0 + sqrt(30.0)) / 36.0, wc = (18.0 - sqrt(30.0)) / 36.0;
    gp[0] = 0.5 - 0.5 * c; gp[1] = 0.5 - 0.5 * a; gp[2] = 0.5 + 0.5 * a; gp[3] = 0.5 + 0.5 * c;
    gw[0] = gw[3] = 0.5 * wc; gw[1] = gw[2] = 0.5 * wa;
  }
  /* cells' local faces by vertex set */
  omap m;
  omap_init(&m, nc * nlf);
  int found;
  int32_t v[4];
  for (int64_t c = 0; c < nc; c++)
    for (int lf = 0; lf < nlf; lf++) {
      for (int i = 0; i < ndv; i++) {
        int lv = ctype == OR_TET4 ? TET_FACES[lf][i] : (D == 2 ? QUAD_EDGES[lf][i] : HEX_FACES[lf][i]);
        v[i] = c_verts[c * nlv + lv - 1];
      }
      int32_t* s = omap_slot(&m, v, ndv, &found);
      if (!found) *s = (int32_t)(c * nlf + lf + 1);
    }
  double val[27], grad[27 * 3], gv[8], gg[8 * 3], be[81];
  int clos[27];
  for (int64_t t = 0; t < nt; t++) {
    int32_t* s = omap_slot(&m, t_verts + t * ndv, ndv, &found);
    if (!found) continue; /* not a face of this mesh */
    const int64_t c = (*s - 1) / nlf;
    const int lf = (int)((*s - 1) % nlf);
    int lvs[4];
    for (int i = 0; i < ndv; i++)
      lvs[i] = (ctype == OR_TET4 ? TET_FACES[lf][i] : (D == 2 ? QUAD_EDGES[lf][i] : HEX_FACES[lf][i])) - 1;
    double X[8 * 3];
    for (int n = 0; n < nlv; n++)
      for (int d = 0; d < D; d++) X[n * D + d] = coords[(int64_t)(cell_nodes[c * nlv + n] - 1) * D + d];
    const int ncl = face_closure_nodes(ctype, order, lf, clos);
    for (int i = 0; i < nloc; i++) be[i] = 0.0;
    const int nq = D == 2 ? n1 : n1 * n1;
    for (int q = 0; q < nq; q++) {
      const double s1 = gp[q % n1], s2 = D == 3 ? gp[q / n1] : 0.0;
      double w = gw[q % n1] * (D == 3 ? gw[q / n1] : 1.0);
      /* reference point xi(s) and its derivatives dxi/ds_a on the face */
      double xi[3] = {0, 0, 0}, dxi[2][3] = {{0, 0, 0}, {0, 0, 0}};
      if (D == 2) {
        for (int d = 0; d < 2; d++) {
          xi[d] = (1.0 - s1) * xv[lvs[0]][d] + s1 * xv[lvs[1]][d];
          dxi[0][d] = xv[lvs[1]][d] - xv[lvs[0]][d];
        }
      } else if (ctype == OR_TET4) {
        const double u = s1, t2 = s2 * (1.0 - s1); /* collapsed coordinates */
        w *= (1.0 - s1);
        for (int d = 0; d < 3; d++) {
          xi[d] = xv[lvs[0]][d] + u * (xv[lvs[1]][d] - xv[lvs[0]][d]) + t2 * (xv[lvs[2]][d] - xv[lvs[0]][d]);
          dxi[0][d] = xv[lvs[1]][d] - xv[lvs[0]][d];
          dxi[1][d] = xv[lvs[2]][d] - xv[lvs[0]][d];
        }
      } else {
        /* square face: its vertices at (0,0), (1,0), (0,1), (1,1) */
        const double N[4] = {(1 - s1) * (1 - s2), s1 * (1 - s2), (1 - s1) * s2, s1 * s2};
        const double dN0[4] = {-(1 - s2), 1 - s2, -s2, s2}, dN1[4] = {-(1 - s1), -s1, 1 - s1, s1};
        for (int d = 0; d < 3; d++)
          for (int i = 0; i < 4; i++) {
            xi[d] += N[i] * xv[lvs[i]][d];
            dxi[0][d] += dN0[i] * xv[lvs[i]][d];
            dxi[1][d] += dN1[i] * xv[lvs[i]][d];
          }
      }
      /* geometry Jacobian at xi, physical tangents T_a = J dxi_a */
      tabulate(ctype, 1, xi, gv, gg);
      double J[9] = {0};
      for (int n = 0; n < nlv; n++)
        for (int i = 0; i < D; i++)
          for (int j = 0; j < D; j++) J[i * D + j] += X[n * D + i] * gg[n * D + j];
      double T[2][3] = {{0, 0, 0}, {0, 0, 0}};
      for (int a = 0; a < D - 1; a++)
        for (int i = 0; i < D; i++)
          for (int j = 0; j < D; j++) T[a][i] += J[i * D + j] * dxi[a][j];
      double meas;
      if (D == 2) {
        meas = sqrt(T[0][0] * T[0][0] + T[0][1] * T[0][1]);
      } else {
        double g11 = 0, g12 = 0, g22 = 0;
        for (int i = 0; i < 3; i++) { g11 += T[0][i] * T[0][i]; g12 += T[0][i] * T[1][i]; g22 += T[1][i] * T[1][i]; }
        meas = sqrt(g11 * g22 - g12 * g12);
      }
      tabulate(ctype, order, xi, val, grad);
      for (int i = 0; i < ncl; i++)
        for (int k = 0; k < ncomp; k++) be[clos[i] * ncomp + k] += g[k] * val[clos[i]] * (meas * w);
    }
    for (int i = 0; i < ncl; i++)
      for (int k = 0; k < ncomp; k++) {
        int32_t dof = cell_dofs[c * nloc + clos[i] * ncomp + k];
        if (dof > 0) b[dof - 1] += be[clos[i] * ncomp + k];
      }
  }
  omap_free(&m);
}

/* Element matrix of one cell (diagnostics / small tests). */
void or_element_matrix(int ctype, int order, int ncomp, int degree, int form, double nu,
                       double coef, const double* X, double* Ke) {
  elem_t e;
  elem_init(&e, ctype, order, ncomp, degree);
  elem_matrix(&e, form, coef, nu, X, Ke);
}

/* ------------------------------------------------------------------------ */
/* Solve checker: Jacobi-preconditioned CG on CSR (0-based).                 */
/* The reference has no CG (it calls an external direct solver,             */
/* src/problems.jl:439-462); this is the FP64 checker for the device CG.     */
/* ------------------------------------------------------------------------ */
int or_pcg(int64_t n, const int64_t* rp, const int32_t* ci, const double* v, const double* b,
           double* x, double rtol, int maxit, double* relres) {
  double *r = malloc(8 * n), *z = malloc(8 * n), *p = malloc(8 * n), *q = malloc(8 * n), *dinv = malloc(8 * n);
  for (int64_t i = 0; i < n; i++) {
    double d = 0.0;
    for (int64_t k = rp[i]; k < rp[i + 1]; k++)
      if (ci[k] == i) d = v[k];
    dinv[i] = 1.0 / d;
  }
  double bn = 0.0;
  for (int64_t i = 0; i < n; i++) {
    double s = 0.0;
    for (int64_t k = rp[i]; k < rp[i + 1]; k++) s += v[k] * x[ci[k]];
    r[i] = b[i] - s;
    bn += b[i] * b[i];
  }
  bn = sqrt(bn);
  if (bn == 0.0) bn = 1.0;
  double rz = 0.0;
  for (int64_t i = 0; i < n; i++) { z[i] = dinv[i] * r[i]; p[i] = z[i]; rz += r[i] * z[i]; }
  int it = 0;
  double rn = 0.0;
  for (int64_t i = 0; i < n; i++) rn += r[i] * r[i];
  rn = sqrt(rn);
  while (rn / bn > rtol && it < maxit) {
    double pq = 0.0;
    for (int64_t i = 0; i < n; i++) {
      double s = 0.0;
      for (int64_t k = rp[i]; k < rp[i + 1]; k++) s += v[k] * p[ci[k]];
      q[i] = s;
      pq += p[i] * s;
    }
    double alpha = rz / pq, rz2 = 0.0;
    rn = 0.0;
    for (int64_t i = 0; i < n; i++) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      z[i] = dinv[i] * r[i];
      rz2 += r[i] * z[i];
      rn += r[i] * r[i];
    }
    rn = sqrt(rn);
    double beta = rz2 / rz;
    rz = rz2;
    for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
    it++;
  }
  *relres = rn / bn;
  free(r); free(z); free(p); free(q); free(dinv);
  return it;
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Threads of the OpenMP loops (1 = the reference's single-threaded path). */
void or_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
