"""gt_assemble_csr (assembly returning the host CSR in one call, with the
pattern download and the input uploads on the copy stream) and the
asynchronous coordinate upload: results bitwise equal to the separate
assemble + download calls."""
import ctypes as C

import numpy as np
import pytest
import torch

import gtgpu as GT
from gtgpu import _lib
from gtgpu.api import _ptr

pytestmark = pytest.mark.gpu


def _space(kind):
    if kind == "p1tet":
        m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (6, 5, 4), simplexify=True)
        GT.jitter_interior_nodes(m, 0.2, 3)
        return m, GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m)), GT.laplacian, 1.0
    if kind == "p1tet_large":
        # 24^3 x 6 cells: the element stage runs in cell chunks and each row
        # chunk's scatter waits only for the chunks holding its rows' cells
        m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (24, 24, 24), simplexify=True)
        GT.jitter_interior_nodes(m, 0.2, 4)
        return m, GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m)), GT.laplacian, 1.0
    if kind == "p2tet":
        # tetrahedra whose elements run in one launch: it waits for the whole
        # (chunked) coefficient upload
        m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (12, 10, 9), simplexify=True)
        GT.jitter_interior_nodes(m, 0.2, 5)
        return m, GT.lagrange_space(GT.interior(m), 2, dirichlet_boundary=GT.boundary(m)), GT.laplacian, 1.0
    if kind == "q1quad":
        m = GT.cartesian_mesh((0, 1, 0, 1), (9, 7))
        return m, GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m)), GT.laplacian, 1.0
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (3, 2, 3))
    V = GT.lagrange_space(GT.interior(m), 2, tensor_size=(3,), dirichlet_boundary=GT.boundary(m, ["2-face-5"]))
    return m, V, (lambda k: GT.elasticity(k, 0.3)), [0.0, 0.0, -1.0]


@pytest.mark.parametrize("kind", ["p1tet", "p1tet_large", "p2tet", "q1quad", "q2hex_elast"])
@pytest.mark.parametrize("pinned", [True, False])
def test_assemble_csr_matches_separate_calls(kind, pinned):
    m, V, form, f = _space(kind)
    kappa = GT.lognormal_cells(m.num_cells, 0.5, 9)
    a = form(kappa)
    A, b = GT.assemble_matrix_and_vector(a, GT.source(f), np.float64, V)
    rp, ci, v = A.csr()
    n, nnz = rp.size - 1, ci.size
    mk = (lambda t, d: torch.empty(t, dtype=d).pin_memory()) if pinned else (lambda t, d: torch.empty(t, dtype=d))
    rp_h, ci_h, v_h, b_h = mk(n + 1, torch.int64), mk(nnz, torch.int32), mk(nnz, torch.float64), mk(n, torch.float64)
    kap = torch.from_numpy(kappa)
    kap = kap.pin_memory() if pinned else kap
    fv = np.ascontiguousarray(np.broadcast_to(np.asarray(f, np.float64), (V.ncomp,)))
    h = C.c_void_p()
    lib = V.ctx.lib
    _lib.check(V.ctx.h, lib.gt_assemble_csr(V.h, a.kind, _ptr(kap), a.nu, _lib.GT_FP64, _ptr(fv), None, _ptr(b_h), nnz,
                                            _ptr(rp_h), _ptr(ci_h), _ptr(v_h), None, C.byref(h)))
    lib.gt_matrix_destroy(h)
    assert np.array_equal(rp_h.numpy(), rp) and np.array_equal(ci_h.numpy(), ci)
    assert np.array_equal(v_h.numpy(), v) and np.array_equal(b_h.numpy(), b)


@pytest.mark.parametrize("prec", ["fp32", "mixed"])
def test_assemble_csr_fp32_and_mixed_values(prec):
    """The pipelined host-buffer path (element chunks, row-chunk scatter,
    chunked downloads) with FP32 values (FP32) or both copies (mixed): the
    values of the separate assembly, bitwise."""
    m, V, form, f = _space("p1tet_large")
    kappa = GT.lognormal_cells(m.num_cells, 0.5, 21)
    a = form(kappa)
    T = np.float32 if prec == "fp32" else "mixed"
    A, b = GT.assemble_matrix_and_vector(a, GT.source(f), T, V)
    rp, ci, _ = A.csr()
    v32 = A.values32()
    n, nnz = rp.size - 1, ci.size
    pin = lambda t, d: torch.empty(t, dtype=d).pin_memory()
    rp_h, ci_h, b_h = pin(n + 1, torch.int64), pin(nnz, torch.int32), pin(n, torch.float64)
    v32_h = pin(nnz, torch.float32)
    v64_h = pin(nnz, torch.float64) if prec == "mixed" else None
    kap = torch.from_numpy(kappa).pin_memory()
    fv = np.ones(1)
    h = C.c_void_p()
    lib = V.ctx.lib
    p = _lib.GT_FP32 if prec == "fp32" else _lib.GT_MIXED
    _lib.check(V.ctx.h, lib.gt_assemble_csr(V.h, a.kind, _ptr(kap), a.nu, p, _ptr(fv), None, _ptr(b_h), nnz,
                                            _ptr(rp_h), _ptr(ci_h), _ptr(v64_h), _ptr(v32_h), C.byref(h)))
    lib.gt_matrix_destroy(h)
    assert np.array_equal(rp_h.numpy(), rp) and np.array_equal(ci_h.numpy(), ci)
    assert np.array_equal(v32_h.numpy(), v32) and np.array_equal(b_h.numpy(), b)
    if prec == "mixed":
        assert np.array_equal(v64_h.numpy(), A.csr()[2])


def test_assemble_csr_capacity_too_small():
    m, V, form, f = _space("q1quad")
    A = GT.assemble_matrix(form(None), np.float64, V, V)
    nnz = A.nnz
    rp = np.zeros(V.num_free_dofs + 1, np.int64)
    ci = np.zeros(nnz, np.int32)
    h = C.c_void_p()
    st = V.ctx.lib.gt_assemble_csr(V.h, _lib.GT_LAPLACE, None, 0.3, _lib.GT_FP64, None, None, None, nnz - 1,
                                   _ptr(rp), _ptr(ci), None, None, C.byref(h))
    assert st == _lib.GT_ERR_INVALID


def test_async_coordinate_upload():
    """set_coords from host memory (copy stream) then assembly: the same
    matrix as a mesh created with those coordinates."""
    m, V, form, f = _space("p1tet")
    m2 = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (6, 5, 4), simplexify=True)
    GT.jitter_interior_nodes(m2, 0.15, 17)
    V2 = GT.lagrange_space(GT.interior(m2), 1, dirichlet_boundary=GT.boundary(m2))
    want = GT.assemble_matrix(GT.laplacian(None), np.float64, V2, V2).csr()[2]
    for pinned in (False, True):
        src = torch.from_numpy(np.ascontiguousarray(m2.coords))
        V.dmesh.set_coords(src.pin_memory() if pinned else src)
        got = GT.assemble_matrix(GT.laplacian(None), np.float64, V, V).csr()[2]
        assert np.array_equal(got, want)
