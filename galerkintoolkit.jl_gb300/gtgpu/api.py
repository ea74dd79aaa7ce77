"""GT-style host API over the C ABI (the drop-in for the assembly + solve path).

Mirrors the problem-level entry points of GalerkinToolkit.jl v0.6.3:

  GT.interior / GT.boundary            src/mesh.jl:223-271
  GT.lagrange_space                    src/space.jl:1702-1735
  GT.assemble_matrix / update_matrix!  src/problems.jl:319-361
  GT.assemble_vector                   src/problems.jl:244-274
  GT.assemble_matrix_and_vector        src/problems.jl:391-414
  GT.update_matrix_and_vector!         src/problems.jl:409-414
  GT.PartitionedSolvers_linear_problem src/problems.jl:439-462 (+ PS.solve)

Weak forms are passed as explicit tags (``laplacian``, ``mass``,
``elasticity``, ``source``) instead of closures; any other form raises
``NotImplementedError`` -- the GB300 kernels implement only these integrands.
Every computation runs in libgtgpu.so on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import GTError, check
from .mesh import Mesh

_default_ctx = None


class Context:
    """Owns a CUDA stream and the device buffer pool (gt_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        st = self.lib.gt_ctx_create(device, C.byref(h))
        if st != 0:
            raise GTError(st, f"gt_ctx_create(device={device}) failed (is a CUDA GPU present?)")
        self.h = h
        self.device = device

    def synchronize(self):
        check(self.h, self.lib.gt_ctx_synchronize(self.h))

    def set_stream(self, stream_ptr):
        check(self.h, self.lib.gt_ctx_set_stream(self.h, stream_ptr))

    def memory(self):
        a, b = C.c_int64(), C.c_int64()
        check(self.h, self.lib.gt_ctx_memory(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def trim(self):
        """Return the context's pooled device blocks to the driver."""
        check(self.h, self.lib.gt_ctx_trim(self.h))

    def launches(self) -> int:
        n = C.c_int64()
        check(self.h, self.lib.gt_ctx_launch_count(self.h, C.byref(n)))
        return n.value

    def graph_launches(self) -> int:
        """CUDA-graph launches so far (each replays a chunk of CG iterations)."""
        n = C.c_int64()
        check(self.h, self.lib.gt_ctx_graph_launch_count(self.h, C.byref(n)))
        return n.value

    def fma_rate(self, fp64=True) -> float:
        """Measured FMA throughput (TFLOP/s) of FP64 or FP32 on this device."""
        t = C.c_double()
        check(self.h, self.lib.gt_ctx_fma_rate(self.h, _lib.GT_FP64 if fp64 else _lib.GT_FP32, C.byref(t)))
        return t.value

    def profile_begin(self):
        check(self.h, self.lib.gt_ctx_profile_begin(self.h))

    def profile_end(self, max_phases=64):
        names = C.create_string_buffer(32 * max_phases)
        ms = np.zeros(max_phases, np.float64)
        n = C.c_int()
        check(self.h, self.lib.gt_ctx_profile_end(self.h, max_phases, names, _ptr(ms), C.byref(n)))
        raw = names.raw
        return [(raw[32 * i:32 * i + 32].split(b"\0")[0].decode(), float(ms[i])) for i in range(n.value)]

    def close(self):
        if self.h:
            self.lib.gt_ctx_destroy(self.h)
            self.h = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _ptr(a):
    """Pointer of a numpy array or a torch tensor (host or device).  The
    caller keeps the array referenced until the C call returns: ctypes
    releases the GIL during the call, so a temporary's memory could be reused
    by another thread meanwhile."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return C.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    raise TypeError(f"unsupported buffer type {type(a)}")


# ---------------------------------------------------------------------------
# mesh on the device
# ---------------------------------------------------------------------------
class DeviceMesh:
    """gt_mesh handle.  Holds no reference back to the host Mesh (which caches
    it), so no reference cycle decides the destruction order."""

    def __init__(self, mesh: Mesh, ctx: Context):
        self.ctx = ctx
        h = C.c_void_p()
        m = mesh
        check(ctx.h, ctx.lib.gt_mesh_create(
            ctx.h, m.cell_type, m.num_nodes, _ptr(m.coords), m.num_cells, _ptr(m.cell_nodes),
            m.corners.size, _ptr(m.corners), m.bfaces.shape[0], _ptr(m.bfaces), _ptr(m.bface_group),
            m.bedges.shape[0], _ptr(m.bedges), C.byref(h)))
        self.h = h

    def set_coords(self, coords):
        check(self.ctx.h, self.ctx.lib.gt_mesh_set_coords(self.h, _ptr(coords)))

    def __del__(self):
        try:
            if self.h and self.ctx.h:
                self.ctx.lib.gt_mesh_destroy(self.h)
        except Exception:
            pass


class DeviceArray:
    """float64 device array from a context's buffer pool (gt_device_alloc):
    a per-cell coefficient or load data that stays on the device.  Passed to
    the forms like a host array; numpy() copies it back."""

    def __init__(self, ctx: Context, n: int):
        self.ctx, self.n = ctx, int(n)
        h = C.c_void_p()
        check(ctx.h, ctx.lib.gt_device_alloc(ctx.h, 8 * self.n, C.byref(h)))
        self.h = h

    def data_ptr(self):
        return self.h.value

    def __len__(self):
        return self.n

    def numpy(self):
        out = np.empty(self.n, np.float64)
        check(self.ctx.h, self.ctx.lib.gt_device_copy(self.ctx.h, _ptr(out), self.h, 8 * self.n))
        return out

    def __del__(self):
        try:
            if self.h and self.ctx.h:
                self.ctx.lib.gt_device_free(self.ctx.h, self.h)
        except Exception:
            pass


def lognormal_cells_device(ncells: int, sigma: float, seed: int, ctx: Context | None = None) -> DeviceArray:
    """The seeded per-cell coefficient of gtgpu.lognormal_cells generated on
    the device (gt_lognormal_cells): same keyed uniforms and Box-Muller
    transform, values equal up to the last bits of log, cos and exp."""
    ctx = ctx or default_context()
    a = DeviceArray(ctx, ncells)
    check(ctx.h, ctx.lib.gt_lognormal_cells(ctx.h, int(ncells), float(sigma), int(seed) & 0xFFFFFFFFFFFFFFFF, a.h))
    return a


def device_mesh(mesh: Mesh, ctx: Context | None = None) -> DeviceMesh:
    ctx = ctx or default_context()
    dm = mesh._device.get(id(ctx))
    if dm is None:
        dm = DeviceMesh(mesh, ctx)
        mesh._device[id(ctx)] = dm
    return dm


# ---------------------------------------------------------------------------
# domains and spaces
# ---------------------------------------------------------------------------
@dataclass
class Domain:
    mesh: Mesh
    dim: int
    group_names: tuple | None = None  # None = every boundary face

    def groups(self):
        """-1 (all boundary faces) or the list of k of "(D-1)-face-k"."""
        if self.group_names is None or "boundary" in self.group_names:
            return -1, None
        ks = []
        for name in self.group_names:
            d, sep, k = name.partition("-face-")
            if not sep or int(d) != self.mesh.D - 1:
                raise ValueError(f"unknown boundary group {name!r}")
            ks.append(int(k))
        return len(ks), np.asarray(ks, np.int32)


def interior(mesh: Mesh) -> Domain:
    return Domain(mesh, mesh.D)


def boundary(mesh: Mesh, group_names=None) -> Domain:
    return Domain(mesh, mesh.D - 1, tuple(group_names) if group_names else None)


class Space:
    """A Lagrange space with device DOF numbering (gt_space)."""

    def __init__(self, domain: Domain, order: int, tensor_size=None, dirichlet_boundary: Domain | None = None,
                 ctx: Context | None = None):
        if domain.dim != domain.mesh.D:
            raise NotImplementedError("spaces live on the interior of the mesh")
        self.ctx = ctx or default_context()
        self.mesh = domain.mesh
        self.dmesh = device_mesh(self.mesh, self.ctx)
        ncomp = 1
        if tensor_size is not None:
            ts = tuple(tensor_size) if not isinstance(tensor_size, int) else (tensor_size,)
            if len(ts) != 1:
                raise NotImplementedError("only scalar and vector spaces are supported")
            ncomp = ts[0]
        if dirichlet_boundary is None:
            ng, groups = 0, None
        else:
            ng, groups = dirichlet_boundary.groups()
        h = C.c_void_p()
        check(self.ctx.h, self.ctx.lib.gt_space_create(self.dmesh.h, order, ncomp, ng, _ptr(groups), C.byref(h)))
        self.h = h
        self.order, self.ncomp = order, ncomp
        info = np.zeros(6, np.int64)
        check(self.ctx.h, self.ctx.lib.gt_space_info(h, _ptr(info)))
        self.num_free_dofs = int(info[0])
        self.num_dirichlet_dofs = int(info[1])
        self.num_local_dofs = int(info[2])

    def node_coordinates(self):
        """Physical coordinates of the space's nodes, ``(free, dirichlet)``
        arrays of shape (nodes, D) in the free and the Dirichlet node
        numbering: the geometry map of each cell (tets: affine; QUAD4/HEX8:
        multilinear) at the reference Lagrange nodes (exponents / order,
        first index fastest; P: exponent sums <= order) -- the points at which
        the reference interpolates Dirichlet data (src/space.jl:1127-1177)."""
        m, D, nc = self.mesh, self.mesh.D, self.ncomp
        cd = self.face_dofs()
        first = cd[:, ::nc]  # component 0 of every local node
        nd = np.where(first > 0, (first - 1) // nc + 1, -((-first - 1) // nc + 1))
        nn = nd.shape[1]
        X = m.coords[m.cell_nodes.astype(np.int64) - 1]  # (cells, vertices, D)
        if m.cell_type == _lib.GT_TET4:
            if self.order == 1:
                N = np.eye(4)
            else:
                # P2 nodes: exponents (a, b, c), a + b + c <= 2, first index
                # fastest; node at (a, b, c) / 2, barycentric weights of the vertices
                ex = [(a, b, c) for c in range(3) for b in range(3) for a in range(3) if a + b + c <= 2]
                P = np.array(ex, np.float64) / 2.0
                N = np.column_stack([1.0 - P.sum(axis=1), P[:, 0], P[:, 1], P[:, 2]])  # (10, 4)
        else:
            k = self.order
            e = np.array(np.unravel_index(np.arange(nn), (k + 1,) * D, order="F")).T / k  # (nn, D)
            nv = 1 << D
            bits = np.array([[(v >> d) & 1 for d in range(D)] for v in range(nv)])  # (nv, D)
            N = np.prod(np.where(bits[None, :, :] == 1, e[:, None, :], 1.0 - e[:, None, :]), axis=2)  # (nn, nv)
        Xn = np.einsum("av,cvd->cad", N, X)
        free = np.zeros((self.num_free_dofs // nc, D))
        diri = np.zeros((self.num_dirichlet_dofs // nc, D))
        f, d = nd > 0, nd < 0
        free[nd[f] - 1] = Xn[f]
        diri[-nd[d] - 1] = Xn[d]
        return free, diri

    def face_dofs(self) -> np.ndarray:
        """GT.face_dofs(V): (ncells, nloc) int32, free > 0, Dirichlet < 0."""
        out = np.zeros((self.mesh.num_cells, self.num_local_dofs), np.int32)
        check(self.ctx.h, self.ctx.lib.gt_space_cell_dofs(self.h, _ptr(out)))
        return out

    def __del__(self):
        try:
            if self.h and self.ctx.h:
                self.ctx.lib.gt_space_destroy(self.h)
        except Exception:
            pass


def lagrange_space(domain: Domain, order: int, tensor_size=None, dirichlet_boundary=None, ctx=None) -> Space:
    return Space(domain, order, tensor_size, dirichlet_boundary, ctx)


def num_free_dofs(V: Space) -> int:
    return V.num_free_dofs


def num_dirichlet_dofs(V: Space) -> int:
    return V.num_dirichlet_dofs


# ---------------------------------------------------------------------------
# weak forms (the supported set)
# ---------------------------------------------------------------------------
@dataclass
class Form:
    kind: int
    coef: object = None    # None, scalar, or per-cell array (host/device)
    nu: float = 0.3

    def cell_coef(self, ncells):
        if self.coef is None:
            return None
        if np.isscalar(self.coef):
            return np.full(ncells, float(self.coef))
        return self.coef


def laplacian(coef=None) -> Form:
    """a(u,v) = int coef grad(u).grad(v) dOmega (per-cell coef)."""
    return Form(_lib.GT_LAPLACE, coef)


def mass(coef=None) -> Form:
    """a(u,v) = int coef u v dOmega."""
    return Form(_lib.GT_MASS, coef)


def elasticity(E=None, nu=0.3) -> Form:
    """a(u,v) = int sigma(eps(u)):eps(v), sigma = lam tr(eps) I + 2 mu eps."""
    return Form(_lib.GT_ELASTICITY, E, float(nu))


@dataclass
class Source:
    f: object = 1.0        # scalar or ncomp vector
    coef: object = None    # optional per-cell factor

    def fvec(self, ncomp):
        return np.ascontiguousarray(np.broadcast_to(np.asarray(self.f, np.float64), (ncomp,)))


def source(f=1.0, coef=None) -> Source:
    """l(v) = int coef f . v dOmega."""
    return Source(f, coef)


def _check_form(a):
    if not isinstance(a, Form):
        raise NotImplementedError("only the Laplacian, mass and linear-elasticity forms are supported "
                                  "on the GPU path (use gtgpu.laplacian / mass / elasticity)")


def _precision(T):
    if T in (np.float64, float, "float64", "fp64"):
        return _lib.GT_FP64
    if T in (np.float32, "float32", "fp32"):
        return _lib.GT_FP32
    if T in ("mixed",):
        return _lib.GT_MIXED
    raise ValueError(f"unsupported value type {T!r}")


# ---------------------------------------------------------------------------
# matrices
# ---------------------------------------------------------------------------
class Matrix:
    """Free x free matrix on the device (block CSR, block = ncomp)."""

    def __init__(self, space: Space, handle, form: Form):
        self.space, self.h, self.form = space, handle, form
        self.ctx = space.ctx
        info = np.zeros(6, np.int64)
        check(self.ctx.h, self.ctx.lib.gt_matrix_info(handle, _ptr(info)))
        self.shape = (int(info[0]), int(info[0]))
        self.nnz = int(info[1])
        self.block_size = int(info[2])
        self.precision = int(info[3])

    def csr(self, dtype=np.float64):
        """(rowptr int64, colind int32, values) of the scalar CSR matrix."""
        n, nnz = self.shape[0], self.nnz
        rp = np.zeros(n + 1, np.int64)
        ci = np.zeros(nnz, np.int32)
        v64 = np.zeros(nnz, np.float64) if dtype == np.float64 and self.precision != _lib.GT_FP32 else None
        v32 = np.zeros(nnz, np.float32) if v64 is None else None
        check(self.ctx.h, self.ctx.lib.gt_matrix_download_csr(self.h, _ptr(rp), _ptr(ci), _ptr(v64), _ptr(v32)))
        return rp, ci, (v64 if v64 is not None else v32)

    def values32(self):
        nnz = self.nnz
        v32 = np.zeros(nnz, np.float32)
        check(self.ctx.h, self.ctx.lib.gt_matrix_download_csr(self.h, None, None, None, _ptr(v32)))
        return v32

    def tocsr(self):
        import scipy.sparse as sp
        rp, ci, v = self.csr()
        return sp.csr_matrix((v, ci, rp), shape=self.shape)

    def __matmul__(self, x):
        y = np.zeros(self.shape[0], np.float64)
        x = np.ascontiguousarray(x, np.float64)
        check(self.ctx.h, self.ctx.lib.gt_spmv(self.h, _ptr(x), _ptr(y)))
        return y

    def __del__(self):
        try:
            if self.h and self.ctx.h:
                self.ctx.lib.gt_matrix_destroy(self.h)
        except Exception:
            pass


def assemble_matrix(a: Form, T, U: Space, V: Space | None = None, reuse=False):
    """GT.assemble_matrix(a, T, U, V): sparsity + values on the GPU."""
    _check_form(a)
    V = V or U
    if V is not U:
        raise NotImplementedError("trial and test spaces must be the same space")
    h = C.c_void_p()
    coef = a.cell_coef(U.mesh.num_cells)
    check(U.ctx.h, U.ctx.lib.gt_assemble_matrix(U.h, a.kind, _ptr(coef), a.nu, _precision(T), C.byref(h)))
    A = Matrix(U, h, a)
    return (A, A) if reuse else A


def update_matrix(A: Matrix, a: Form | None = None):
    """GT.update_matrix!(A, cache): new values on the same sparsity."""
    a = a or A.form
    _check_form(a)
    coef = a.cell_coef(A.space.mesh.num_cells)
    check(A.ctx.h, A.ctx.lib.gt_update_matrix(A.h, a.kind, _ptr(coef), a.nu))
    A.form = a
    return A


def update_matrix_and_vector(A: Matrix, a: Form, l: Source, out=None):
    """GT.update_matrix_and_vector! (src/problems.jl:409-414): new matrix
    values and load vector on A's sparsity, bitwise what a fresh
    assemble_matrix_and_vector of the same forms gives."""
    _check_form(a)
    if not isinstance(l, Source):
        raise NotImplementedError("only source terms int coef*f*v are supported")
    V = A.space
    b = out if out is not None else np.zeros(V.num_free_dofs, np.float64)
    coef = a.cell_coef(V.mesh.num_cells)
    scoef = None if l.coef is None else (np.full(V.mesh.num_cells, float(l.coef)) if np.isscalar(l.coef) else l.coef)
    fv = l.fvec(V.ncomp)  # kept alive across the call (ctypes releases the GIL)
    check(A.ctx.h, A.ctx.lib.gt_update_matrix_and_vector(A.h, a.kind, _ptr(coef), a.nu, _ptr(fv), _ptr(scoef), _ptr(b)))
    A.form = a
    return A, b


def assemble_vector(l: Source, T, V: Space, out=None):
    """GT.assemble_vector(l, T, V) for l(v) = int coef f . v."""
    if not isinstance(l, Source):
        raise NotImplementedError("only source terms int coef*f*v are supported (use gtgpu.source)")
    b = out if out is not None else np.zeros(V.num_free_dofs, np.float64)
    coef = None if l.coef is None else (np.full(V.mesh.num_cells, float(l.coef)) if np.isscalar(l.coef) else l.coef)
    fv = l.fvec(V.ncomp)  # kept alive across the call (ctypes releases the GIL)
    check(V.ctx.h, V.ctx.lib.gt_assemble_vector(V.h, _ptr(fv), _ptr(coef), _ptr(b)))
    return b


def assemble_boundary_vector(g, gamma: Domain, V: Space, out=None, accumulate=False):
    """GT.assemble_vector(v -> int g v dGamma, T, V) over the boundary faces
    of gamma (boundary(mesh, groups)): the Neumann term, g a constant (or
    ncomp constants on a vector space).  With accumulate, adds to out."""
    if gamma.dim != V.mesh.D - 1:
        raise NotImplementedError("boundary integrals over the (D-1)-faces of the boundary only")
    ng, groups = gamma.groups()
    gv = np.ascontiguousarray(np.broadcast_to(np.asarray(g, np.float64), (V.ncomp,)))
    b = out if out is not None else np.zeros(V.num_free_dofs, np.float64)
    check(V.ctx.h, V.ctx.lib.gt_assemble_boundary_vector(V.h, ng, _ptr(groups), _ptr(gv), _ptr(b),
                                                         1 if accumulate else 0))
    return b


def assemble_matrix_and_vector(a: Form, l: Source, T, U: Space, V: Space | None = None, out=None):
    """GT.assemble_matrix_and_vector(a, l, T, U, V) -> (A, b)."""
    _check_form(a)
    if not isinstance(l, Source):
        raise NotImplementedError("only source terms int coef*f*v are supported")
    V = V or U
    if V is not U:
        raise NotImplementedError("trial and test spaces must be the same space")
    h = C.c_void_p()
    b = out if out is not None else np.zeros(U.num_free_dofs, np.float64)
    coef = a.cell_coef(U.mesh.num_cells)
    scoef = None if l.coef is None else (np.full(U.mesh.num_cells, float(l.coef)) if np.isscalar(l.coef) else l.coef)
    fv = l.fvec(U.ncomp)  # kept alive across the call (ctypes releases the GIL)
    check(U.ctx.h, U.ctx.lib.gt_assemble_matrix_and_vector(U.h, a.kind, _ptr(coef), a.nu, _precision(T),
                                                           _ptr(fv), _ptr(scoef), _ptr(b), C.byref(h)))
    return Matrix(U, h, a), b


# ---------------------------------------------------------------------------
# linear problems and the solve
# ---------------------------------------------------------------------------
@dataclass
class LinearProblem:
    A: Matrix
    b: np.ndarray
    x: np.ndarray


def interpolate_dirichlet(g, V: Space) -> np.ndarray:
    """GT.interpolate_dirichlet(g, V): the Dirichlet values of the function
    g at the space's Dirichlet nodes, in the Dirichlet DOF numbering (DOF -k
    -> xd[k-1]).  g maps an (n, D) array of points to (n,) values or, on a
    vector space, to (n, ncomp)."""
    _, xdir = V.node_coordinates()
    vals = np.asarray(g(xdir), np.float64)
    if V.ncomp == 1:
        vals = vals.reshape(-1)
    else:
        vals = vals.reshape(-1, V.ncomp)
    return np.ascontiguousarray(vals.reshape(-1))


class Polynomial:
    """A quadratic p(x) = c0 + cx x + cy y + cz z + cxx x^2 + cyy y^2 + czz z^2
    + cxy xy + cxz xz + cyz yz: the exact solutions of the reference's patch
    tests (u = x + y, test/assembly_tests.jl:43-118) and the integrands of its
    integration tests.  Callable on an (n, D) array of points, so it also
    serves as Dirichlet data for interpolate_dirichlet."""

    NAMES = ("c0", "x", "y", "z", "xx", "yy", "zz", "xy", "xz", "yz")

    def __init__(self, c0=0.0, x=0.0, y=0.0, z=0.0, xx=0.0, yy=0.0, zz=0.0, xy=0.0, xz=0.0, yz=0.0):
        self.c = np.array([c0, x, y, z, xx, yy, zz, xy, xz, yz], np.float64)

    def __call__(self, X):
        X = np.asarray(X, np.float64)
        P = np.zeros((X.shape[0], 3))
        P[:, :X.shape[1]] = X
        x, y, z = P[:, 0], P[:, 1], P[:, 2]
        c = self.c
        return (c[0] + c[1] * x + c[2] * y + c[3] * z + c[4] * x * x + c[5] * y * y + c[6] * z * z + c[7] * x * y
                + c[8] * x * z + c[9] * y * z)


class DiscreteField:
    """GT.DiscreteField of a Lagrange space (src/field.jl): the free DOF
    values and the Dirichlet DOF values (DOF -k -> dirichlet_values[k-1]).
    ``integrate`` / ``l2_error`` / ``h1_error`` take one in place of the
    (uh, dirichlet_values) pair."""

    def __init__(self, space: Space, free_values, dirichlet_values):
        fv = np.ascontiguousarray(free_values, np.float64)
        dv = np.ascontiguousarray(dirichlet_values, np.float64)
        if fv.size != space.num_free_dofs:
            raise ValueError(f"{fv.size} free values, the space has {space.num_free_dofs} free DOFs")
        if dv.size != space.num_dirichlet_dofs:
            raise ValueError(f"{dv.size} Dirichlet values, the space has {space.num_dirichlet_dofs} Dirichlet DOFs")
        self.space, self.free_values, self.dirichlet_values = space, fv, dv

    def dof_values(self) -> np.ndarray:
        """Values per cell and local DOF, (ncells, nloc): free DOF d > 0 takes
        free_values[d-1], Dirichlet DOF -k takes dirichlet_values[k-1]."""
        cd = self.space.face_dofs().astype(np.int64)
        out = np.empty(cd.shape, np.float64)
        f = cd > 0
        out[f] = self.free_values[cd[f] - 1]
        out[~f] = self.dirichlet_values[-cd[~f] - 1]
        return out


def zero_dirichlet_field(U: Space) -> DiscreteField:
    """GT.zero_dirichlet_field(T, U): zero free and Dirichlet values."""
    return DiscreteField(U, np.zeros(U.num_free_dofs), np.zeros(U.num_dirichlet_dofs))


def dirichlet_field(U: Space, g=None) -> DiscreteField:
    """The Dirichlet field uhd of GT.interpolate_dirichlet!(g, uhd)
    (src/field.jl:364-367): zero free values, Dirichlet values of g at the
    Dirichlet nodes (zero without g)."""
    xd = np.zeros(U.num_dirichlet_dofs) if g is None else interpolate_dirichlet(g, U)
    return DiscreteField(U, np.zeros(U.num_free_dofs), xd)


def solution_field(U, x) -> DiscreteField:
    """GT.solution_field (src/problems.jl:501-516): the discrete field with
    free values x (a vector, or the solution of a LinearProblem) and the
    Dirichlet values of uhd -- ``solution_field(uhd, x)`` -- or zero Dirichlet
    values -- ``solution_field(U, x)``."""
    if isinstance(x, LinearProblem):
        x = x.x
    if isinstance(U, DiscreteField):
        return DiscreteField(U.space, np.array(x, np.float64, copy=True), U.dirichlet_values.copy())
    return DiscreteField(U, np.array(x, np.float64, copy=True), np.zeros(U.num_dirichlet_dofs))


def solution_field_inplace(uh: DiscreteField, x) -> DiscreteField:
    """GT.solution_field!(uh, x) (src/problems.jl:518-526): new free values,
    the Dirichlet values kept."""
    if isinstance(x, LinearProblem):
        x = x.x
    x = np.asarray(x, np.float64)
    if x.size != uh.free_values.size:
        raise ValueError(f"{x.size} values, the field has {uh.free_values.size} free DOFs")
    uh.free_values[...] = x
    return uh


_INT_KINDS = {"volume": _lib.GT_INT_VOLUME, "poly": _lib.GT_INT_POLY, "field": _lib.GT_INT_FIELD,
              "l2_norm2": _lib.GT_INT_L2_NORM2, "l2_error2": _lib.GT_INT_L2_ERROR2, "h1_error2": _lib.GT_INT_H1_ERROR2}


def integrate(V: Space, kind="volume", uh=None, exact=None, dirichlet_values=None) -> float:
    """GT.assemble_scalar (src/problems.jl:172-190) for fixed integrands over
    the cells of V's mesh: "volume" (int 1), "poly" (int p, exact a
    Polynomial), "field" (int sum_k u_k), "l2_norm2" (int |u|^2),
    "l2_error2" (int |u - p|^2) and "h1_error2" (int |grad u - grad p|^2).  uh:
    a DiscreteField, or the free DOF values (e.g. a solution) with
    dirichlet_values the Dirichlet DOF values (default 0); exact: a
    Polynomial, or one per component."""
    k = _INT_KINDS[kind]
    if isinstance(uh, DiscreteField):
        uh, dirichlet_values = uh.free_values, uh.dirichlet_values
    uf = None if uh is None else np.ascontiguousarray(uh, np.float64)
    if uf is not None and uf.size != V.num_free_dofs:
        raise ValueError(f"uh has {uf.size} entries, the space has {V.num_free_dofs} free DOFs")
    ud = None if dirichlet_values is None else np.ascontiguousarray(dirichlet_values, np.float64)
    if ud is not None and ud.size != V.num_dirichlet_dofs:
        raise ValueError(f"dirichlet_values has {ud.size} entries, the space has {V.num_dirichlet_dofs}")
    pc = None
    if exact is not None:
        ps = exact if isinstance(exact, (list, tuple)) else [exact] * (1 if kind == "poly" else V.ncomp)
        pc = np.ascontiguousarray(np.concatenate([p.c for p in ps]), np.float64)
    out = C.c_double(0.0)
    check(V.ctx.h, V.ctx.lib.gt_integrate(V.h, k, _ptr(uf), _ptr(ud), _ptr(pc), C.byref(out)))
    return out.value


def l2_error(V: Space, uh, exact, dirichlet_values=None) -> float:
    """sqrt(int |u_h - u|^2) for a polynomial exact solution u (uh: a
    DiscreteField or the free values)"""
    return float(np.sqrt(integrate(V, "l2_error2", uh, exact, dirichlet_values)))


def h1_error(V: Space, uh, exact, dirichlet_values=None) -> float:
    """sqrt(int |grad u_h - grad u|^2) for a polynomial exact solution u (uh:
    a DiscreteField or the free values)"""
    return float(np.sqrt(integrate(V, "h1_error2", uh, exact, dirichlet_values)))


def linear_problem(U: Space, a: Form, l: Source, T=np.float64, V=None, dirichlet_values=None,
                   neumann=None) -> LinearProblem:
    """GT.PartitionedSolvers_linear_problem: A and b assembled on the GPU,
    x = 0.  With dirichlet_values (the Dirichlet field uhd of
    dirichlet_field(U, g), or its values interpolate_dirichlet(g, U)) the
    Dirichlet lift b -= Ad * xd is applied in the same pass
    (src/problems.jl:439-453); without, homogeneous Dirichlet data.
    neumann: (g, boundary(mesh, groups)) pairs whose boundary terms
    int g v dGamma are added to b."""
    if isinstance(dirichlet_values, DiscreteField):
        dirichlet_values = dirichlet_values.dirichlet_values
    lp = _linear_problem(U, a, l, T, V, dirichlet_values)
    for g, gamma in (neumann or ()):
        assemble_boundary_vector(g, gamma, U, out=lp.b, accumulate=True)
    return lp


def _linear_problem(U: Space, a: Form, l: Source, T, V, dirichlet_values) -> LinearProblem:
    if dirichlet_values is None:
        A, b = assemble_matrix_and_vector(a, l, T, U, V)
        return LinearProblem(A, b, np.zeros_like(b))
    _check_form(a)
    if not isinstance(l, Source):
        raise NotImplementedError("only source terms int coef*f*v are supported")
    if V is not None and V is not U:
        raise NotImplementedError("trial and test spaces must be the same space")
    xd = np.ascontiguousarray(dirichlet_values, np.float64)
    if xd.size != U.num_dirichlet_dofs:
        raise ValueError(f"dirichlet_values has {xd.size} entries, the space has {U.num_dirichlet_dofs} Dirichlet DOFs")
    h = C.c_void_p()
    b = np.zeros(U.num_free_dofs, np.float64)
    coef = a.cell_coef(U.mesh.num_cells)
    scoef = None if l.coef is None else (np.full(U.mesh.num_cells, float(l.coef)) if np.isscalar(l.coef) else l.coef)
    fv = l.fvec(U.ncomp)  # kept alive across the call (ctypes releases the GIL)
    check(U.ctx.h, U.ctx.lib.gt_linear_problem(U.h, a.kind, _ptr(coef), a.nu, _precision(T), _ptr(fv), _ptr(scoef),
                                               _ptr(xd), _ptr(b), C.byref(h)))
    return LinearProblem(Matrix(U, h, a), b, np.zeros_like(b))


_MODES = {"fp64": _lib.GT_SOLVE_FP64, "ir": _lib.GT_SOLVE_IR, "mixed": _lib.GT_SOLVE_IR, "fp32": _lib.GT_SOLVE_FP32}


def solve(p: LinearProblem | Matrix, b=None, x=None, rtol=1e-10, maxit=20000, mode="fp64", raise_on_fail=True):
    """Jacobi-PCG (mode "fp64"), FP32 PCG with FP64 reliable updates ("ir" or
    "mixed"), or FP32 PCG ("fp32").  Returns (x, info dict)."""
    if isinstance(p, LinearProblem):
        A, b, x = p.A, p.b, p.x if x is None else x
    else:
        A = p
        x = np.zeros(A.shape[0]) if x is None else x
    info = _lib.SolveInfo()
    st = A.ctx.lib.gt_solve(A.h, _ptr(b), _ptr(x), float(rtol), int(maxit), _MODES[mode], C.byref(info))
    if st != 0 and (raise_on_fail or st != _lib.GT_ERR_NOT_CONVERGED):
        check(A.ctx.h, st)
    return x, dict(iterations=info.iterations, outer_iterations=info.outer_iterations,
                   rel_residual=info.rel_residual, fp64_iterations=info.fp64_iterations, converged=st == 0)
