"""CPU oracle for the finite-element assembly path (TEST INFRASTRUCTURE ONLY).

This module wraps ``gt_oracle.c`` (a C restatement of GalerkinToolkit.jl's
algorithms, compiled by ``oracle/Makefile``) and adds the orchestration the
reference performs between those kernels: mesh -> topology -> DOF ids ->
COO -> CSC.  Only the test-suite, ``__graft_entry__.smoke`` and the CPU-baseline
leg of ``bench.py`` may import it.  The product package never does.

Reference call stack restated here (paths inside GalerkinToolkit.jl v0.6.3):
  cartesian_mesh            src/cartesian_mesh.jl:16-54, :97-461
  complexify / numbering    src/topology.jl:867-1125, :1468-1704
  generate_dof_ids          src/space.jl:299-535
  assemble_matrix           src/problems.jl:319-350 -> src/assembly.jl:75-208,545-575
  assemble_vector           src/problems.jl:244-274 -> src/assembly.jl:27-73,558-569
Parity with the reference is pinned by the reference's own known-answer
tests (re-expressed in tests/test_oracle_known_answers.py); the Julia package
itself cannot run in this environment, so there are no generated fixtures.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgtoracle.so")

QUAD4, HEX8, TET4 = 1, 2, 3
LAPLACE, MASS, ELASTICITY = 1, 2, 3

QUAD_EDGES = np.array([[1, 2], [3, 4], [1, 3], [2, 4]], np.int32)
HEX_EDGES = np.array([[1, 2], [3, 4], [1, 3], [2, 4], [5, 6], [7, 8],
                      [5, 7], [6, 8], [1, 5], [3, 7], [2, 6], [4, 8]], np.int32)
HEX_FACES = np.array([[1, 2, 3, 4], [5, 6, 7, 8], [1, 2, 5, 6],
                      [3, 4, 7, 8], [1, 3, 5, 7], [2, 4, 6, 8]], np.int32)
# unit simplex local faces, src/domain.jl:413-469
TRI_EDGES = np.array([[1, 2], [1, 3], [2, 3]], np.int32)
TET_EDGES = np.array([[1, 2], [1, 3], [2, 3], [1, 4], [2, 4], [3, 4]], np.int32)
TET_FACES = np.array([[1, 2, 3], [1, 2, 4], [1, 3, 4], [2, 3, 4]], np.int32)

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library with ``make`` (gcc, OpenMP)."""
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "gt_oracle.c"))):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB_PATH)
            i64, i32, dbl, u64 = C.c_int64, C.c_int, C.c_double, C.c_uint64
            P = C.c_void_p
            L.or_cartesian_mesh_counts.argtypes = [i32, P, i32, P]
            L.or_cartesian_mesh.argtypes = [i32, P, P, i32, P, P, P, P, P, P, P]
            L.or_jitter_nodes.argtypes = [i32, P, P, dbl, u64, P]
            L.or_lognormal_cells.argtypes = [i64, dbl, u64, P]
            L.or_uniform.argtypes = [u64, u64]
            L.or_uniform.restype = dbl
            L.or_vertex_ids.argtypes = [i64, i64, P, P]
            L.or_vertex_ids.restype = i64
            L.or_face_boundary.argtypes = [i64, i32, P, i32, i32, P, i64, P, P, P]
            L.or_face_boundary.restype = i64
            L.or_face_lookup.argtypes = [i64, i32, P, i32, i32, P, i64, P, P]
            L.or_dof_ids.argtypes = [i32, i32, i32, i64, P, i64, P, i64, P, i64, P, P, P]
            L.or_dof_ids.restype = i64
            L.or_tag_cell_faces.argtypes = [i32, i64, P, i64, P, P]
            L.or_quadrature.argtypes = [i32, i32, P, P]
            L.or_quadrature.restype = i32
            L.or_count_coo.argtypes = [i64, i32, P, i32, P]
            L.or_count_coo.restype = i64
            L.or_fill_coo.argtypes = [i32, i32, i32, i32, i32, dbl, i64, P, P, P, P, i32, P, P, P, P]
            L.or_coo_to_csc.argtypes = [i64, P, P, P, i64, P, P, P]
            L.or_coo_to_csc.restype = i64
            L.or_assemble_vector.argtypes = [i32, i32, i32, i32, P, i64, P, P, P, P, i64, P]
            L.or_element_matrix.argtypes = [i32, i32, i32, i32, i32, dbl, dbl, P, P]
            L.or_pcg.argtypes = [i64, P, P, P, P, P, dbl, i32, P]
            L.or_pcg.restype = i32
            L.or_num_threads.restype = i32
            L.or_set_num_threads.argtypes = [i32]
            L.or_assemble_boundary_vector.argtypes = [i32, i32, i32, i32, P, i64, P, P, P, P, i64, P, P]
            _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# --------------------------------------------------------------------------
# mesh
# --------------------------------------------------------------------------

def cartesian_mesh(box, cells, simplexify=False):
    """cartesian_mesh(domain, cells; simplexify) of the reference (with
    boundary faces and groups).  Returns a dict of numpy arrays (1-based ids)."""
    D = len(cells)
    n = np.asarray(cells, np.int32)
    bx = np.asarray(box, np.float64)
    cnt = np.zeros(8, np.int64)
    L = lib()
    L.or_cartesian_mesh_counts(D, _p(n), int(simplexify), _p(cnt))
    nnodes, ncells, nv = int(cnt[0]), int(cnt[1]), int(cnt[2])
    coords = np.zeros((nnodes, D), np.float64)
    cell_nodes = np.zeros((ncells, nv), np.int32)
    pf0 = np.zeros(int(cnt[3]), np.int32)
    pf1 = np.zeros((int(cnt[4]), 2), np.int32)
    pf1g = np.zeros(int(cnt[4]), np.int32)
    nfv = 3 if simplexify else 4
    npf2 = int(cnt[5]) if D == 3 else 0
    pf2 = np.zeros((npf2, nfv), np.int32)
    pf2g = np.zeros(npf2, np.int32)
    L.or_cartesian_mesh(D, _p(n), _p(bx), int(simplexify), _p(coords), _p(cell_nodes),
                        _p(pf0), _p(pf1), _p(pf1g), _p(pf2), _p(pf2g))
    ctype = TET4 if simplexify else (QUAD4 if D == 2 else HEX8)
    m = dict(D=D, ctype=ctype, cells=tuple(int(c) for c in cells), box=tuple(float(b) for b in box),
             coords=coords, cell_nodes=cell_nodes, pf0=pf0, pf1=pf1, pf1g=pf1g)
    if D == 3:
        m["pf2"], m["pf2g"] = pf2, pf2g
    return m


def jitter(mesh, amp, seed):
    n = np.asarray(mesh["cells"], np.int32)
    bx = np.asarray(mesh["box"], np.float64)
    lib().or_jitter_nodes(mesh["D"], _p(n), _p(bx), float(amp), int(seed), _p(mesh["coords"]))
    return mesh


def lognormal_cells(ncells, sigma, seed):
    out = np.zeros(ncells, np.float64)
    lib().or_lognormal_cells(int(ncells), float(sigma), int(seed), _p(out))
    return out


def boundary_faces(mesh, groups=None):
    """Tagged (D-1)-faces (node ids) of the named groups ("boundary" = all)."""
    D = mesh["D"]
    key, gk = ("pf2", "pf2g") if D == 3 else ("pf1", "pf1g")
    faces, g = mesh[key], mesh[gk]
    if groups is None or groups == "boundary" or groups == ["boundary"]:
        return faces
    ks = []
    for name in groups:
        d, _, k = name.partition("-face-")
        assert int(d) == D - 1, name
        ks.append(int(k))
    return faces[np.isin(g, ks)]


# --------------------------------------------------------------------------
# space: topology + DOF numbering
# --------------------------------------------------------------------------

def lagrange_space(mesh, order, ncomp=1, dirichlet=None):
    """lagrange_space(Omega, order; tensor_size, dirichlet_boundary): cell_dofs
    (1-based free, negative Dirichlet), nfree, ndiri."""
    L = lib()
    D, ctype = mesh["D"], mesh["ctype"]
    coords, cn = mesh["coords"], mesh["cell_nodes"]
    nnodes, nc = coords.shape[0], cn.shape[0]
    node_vertex = np.zeros(nnodes, np.int32)
    nverts = L.or_vertex_ids(nnodes, mesh["pf0"].size, _p(mesh["pf0"]), _p(node_vertex))
    c_verts = np.ascontiguousarray(node_vertex[cn - 1])
    c_edges = c_faces = None
    nedges = nfaces = 0
    if order == 2 and ctype == TET4:
        # triangles over the tets (parents: boundary triangles), edges over the
        # triangles (parents: boundary 1-faces), the tets' edges looked up
        # (create_face_boundary!, src/topology.jl:1099-1125)
        c_faces = np.zeros((nc, 4), np.int32)
        par = np.ascontiguousarray(node_vertex[mesh["pf2"] - 1])
        fv = np.zeros((par.shape[0] + nc * 4, 3), np.int32)
        nfaces = L.or_face_boundary(nc, 4, _p(c_verts), 4, 3, _p(TET_FACES), par.shape[0], _p(par),
                                    _p(c_faces), _p(fv))
        fv = np.ascontiguousarray(fv[:nfaces])
        f_edges = np.zeros((nfaces, 3), np.int32)
        par1 = np.ascontiguousarray(node_vertex[mesh["pf1"] - 1])
        ev = np.zeros((par1.shape[0] + nfaces * 3, 2), np.int32)
        nedges = L.or_face_boundary(nfaces, 3, _p(fv), 3, 2, _p(TRI_EDGES), par1.shape[0], _p(par1),
                                    _p(f_edges), _p(ev))
        ev = np.ascontiguousarray(ev[:nedges])
        c_edges = np.zeros((nc, 6), np.int32)
        L.or_face_lookup(nc, 4, _p(c_verts), 6, 2, _p(TET_EDGES), nedges, _p(ev), _p(c_edges))
        c_faces, nfaces = None, 0  # P2 has no face-interior nodes
    elif order == 2:
        assert ctype in (QUAD4, HEX8)
        if D == 2:
            c_edges = np.zeros((nc, 4), np.int32)
            par = np.ascontiguousarray(node_vertex[mesh["pf1"] - 1])
            ev = np.zeros((par.shape[0] + nc * 4, 2), np.int32)
            nedges = L.or_face_boundary(nc, 4, _p(c_verts), 4, 2, _p(QUAD_EDGES), par.shape[0], _p(par),
                                        _p(c_edges), _p(ev))
        else:
            c_faces = np.zeros((nc, 6), np.int32)
            par = np.ascontiguousarray(node_vertex[mesh["pf2"] - 1])
            fv = np.zeros((par.shape[0] + nc * 6, 4), np.int32)
            nfaces = L.or_face_boundary(nc, 8, _p(c_verts), 6, 4, _p(HEX_FACES), par.shape[0], _p(par),
                                        _p(c_faces), _p(fv))
            fv = np.ascontiguousarray(fv[:nfaces])
            f_edges = np.zeros((nfaces, 4), np.int32)
            par1 = np.ascontiguousarray(node_vertex[mesh["pf1"] - 1])
            ev = np.zeros((par1.shape[0] + nfaces * 4, 2), np.int32)
            nedges = L.or_face_boundary(nfaces, 4, _p(fv), 4, 2, _p(QUAD_EDGES), par1.shape[0], _p(par1),
                                        _p(f_edges), _p(ev))
            ev = np.ascontiguousarray(ev[:nedges])
            c_edges = np.zeros((nc, 12), np.int32)
            L.or_face_lookup(nc, 8, _p(c_verts), 12, 2, _p(HEX_EDGES), nedges, _p(ev), _p(c_edges))
    nlf = 4 if ctype == TET4 else 2 * D
    c_tagged = np.zeros((nc, nlf), np.uint8)
    if dirichlet is not None:
        tf = np.ascontiguousarray(node_vertex[boundary_faces(mesh, dirichlet) - 1])
        L.or_tag_cell_faces(ctype, nc, _p(c_verts), tf.shape[0], _p(tf), _p(c_tagged))
    nn = (10 if order == 2 else 4) if ctype == TET4 else (order + 1) ** D
    cell_dofs = np.zeros((nc, nn * ncomp), np.int32)
    ndiri = np.zeros(1, np.int64)
    nfree = L.or_dof_ids(ctype, order, ncomp, nc, _p(c_verts), nverts, _p(c_edges), nedges,
                         _p(c_faces), nfaces, _p(c_tagged), _p(cell_dofs), _p(ndiri))
    return dict(mesh=mesh, order=order, ncomp=ncomp, cell_dofs=cell_dofs, nfree=int(nfree),
                ndiri=int(ndiri[0]), nverts=int(nverts), nedges=int(nedges), nfaces=int(nfaces),
                node_vertex=node_vertex)


def quadrature(ctype, degree):
    x = np.zeros((27, 3), np.float64)
    w = np.zeros(27, np.float64)
    nq = lib().or_quadrature(ctype, degree, _p(x), _p(w))
    D = 2 if ctype == QUAD4 else 3
    return x.reshape(-1)[: nq * D].reshape(nq, D).copy(), w[:nq].copy()


# --------------------------------------------------------------------------
# assembly
# --------------------------------------------------------------------------

def assemble_coo(space, form, degree, coef=None, nu=0.3, dirichlet_cols=False):
    L = lib()
    mesh = space["mesh"]
    cd = space["cell_dofs"]
    nc, nloc = cd.shape
    off = np.zeros(nc + 1, np.int64)
    n = L.or_count_coo(nc, nloc, _p(cd), int(dirichlet_cols), _p(off))
    I = np.zeros(n, np.int32)
    J = np.zeros(n, np.int32)
    V = np.zeros(n, np.float64)
    coef = None if coef is None else np.ascontiguousarray(coef, np.float64)
    L.or_fill_coo(mesh["ctype"], space["order"], space["ncomp"], degree, form, float(nu), nc,
                  _p(mesh["cell_nodes"]), _p(mesh["coords"]), _p(cd), _p(coef), int(dirichlet_cols),
                  _p(off), _p(I), _p(J), _p(V))
    return I, J, V


def coo_to_csc(I, J, V, ncols):
    n = I.size
    colptr = np.zeros(ncols + 1, np.int64)
    rowval = np.zeros(n, np.int32)
    nzval = np.zeros(n, np.float64)
    nnz = lib().or_coo_to_csc(n, _p(I), _p(J), _p(V), ncols, _p(colptr), _p(rowval), _p(nzval))
    return colptr, rowval[:nnz].copy(), nzval[:nnz].copy()


def assemble_matrix(space, form, degree, coef=None, nu=0.3, dirichlet_cols=False):
    """assemble_matrix(a, Float64, V, V): free x free (or free x Dirichlet)
    SparseMatrixCSC as (colptr, rowval, nzval), 0-based."""
    I, J, V = assemble_coo(space, form, degree, coef, nu, dirichlet_cols)
    ncols = space["ndiri"] if dirichlet_cols else space["nfree"]
    return coo_to_csc(I, J, V, ncols)


def csc_to_csr(colptr, rowval, nzval, nrows):
    """Transpose-free re-layout of a CSC matrix as CSR (rows sorted cols)."""
    ncols = colptr.size - 1
    cols = np.repeat(np.arange(ncols, dtype=np.int32), np.diff(colptr))
    order = np.lexsort((cols, rowval))
    rowptr = np.zeros(nrows + 1, np.int64)
    np.add.at(rowptr, rowval.astype(np.int64) + 1, 1)
    rowptr = np.cumsum(rowptr)
    return rowptr, cols[order].astype(np.int32), nzval[order]


def assemble_vector(space, degree, f, coef=None):
    mesh = space["mesh"]
    cd = space["cell_dofs"]
    b = np.zeros(space["nfree"], np.float64)
    fv = np.ascontiguousarray(np.broadcast_to(np.asarray(f, np.float64), (space["ncomp"],)))
    coef = None if coef is None else np.ascontiguousarray(coef, np.float64)
    lib().or_assemble_vector(mesh["ctype"], space["order"], space["ncomp"], degree, _p(fv), cd.shape[0],
                             _p(mesh["cell_nodes"]), _p(mesh["coords"]), _p(cd), _p(coef), space["nfree"], _p(b))
    return b


def element_matrix(ctype, order, ncomp, degree, form, X, coef=1.0, nu=0.3):
    nloc = (4 if ctype == TET4 else (order + 1) ** (2 if ctype == QUAD4 else 3)) * ncomp
    Ke = np.zeros((nloc, nloc), np.float64)
    X = np.ascontiguousarray(X, np.float64)
    lib().or_element_matrix(ctype, order, ncomp, degree, form, float(nu), float(coef), _p(X), _p(Ke))
    return Ke


def pcg(rowptr, colind, vals, b, rtol=1e-12, maxit=10000):
    x = np.zeros_like(b)
    rr = np.zeros(1)
    it = lib().or_pcg(b.size, _p(rowptr), _p(colind), _p(vals), _p(b), _p(x), float(rtol), int(maxit), _p(rr))
    return x, int(it), float(rr[0])


def num_threads():
    return int(lib().or_num_threads())


def set_threads(n):
    """Threads of the oracle's OpenMP loops (1: the reference's
    single-threaded path)."""
    lib().or_set_num_threads(int(n))


def assemble_boundary_vector(space, degree, g, groups=None):
    """The Neumann term int g . v dGamma (constant g, ncomp values) over the
    boundary faces of the named groups (None / "boundary": all), the loop of
    assemble_in_Γn! (docs/src/src_jl/example_poisson_equation.jl:161-203);
    free DOFs only."""
    mesh = space["mesh"]
    cd = space["cell_dofs"]
    nv = space["node_vertex"]
    c_verts = np.ascontiguousarray(nv[mesh["cell_nodes"] - 1])
    tf = np.ascontiguousarray(nv[boundary_faces(mesh, groups) - 1])
    fv = np.ascontiguousarray(np.broadcast_to(np.asarray(g, np.float64), (space["ncomp"],)))
    b = np.zeros(space["nfree"], np.float64)
    lib().or_assemble_boundary_vector(mesh["ctype"], space["order"], space["ncomp"], int(degree), _p(fv),
                                      cd.shape[0], _p(mesh["cell_nodes"]), _p(mesh["coords"]), _p(cd),
                                      _p(c_verts), tf.shape[0], _p(tf), _p(b))
    return b
