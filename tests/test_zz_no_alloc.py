"""gt_update_matrix_noalloc: the matrix refill that allocates no device memory.

Callers that cannot let the library allocate -- a process whose device memory
is budgeted up front by its own admission control or memory pool, or a
latency-critical refill loop where cudaMalloc/cudaFree would synchronise the
device -- refill an assembled matrix through this entry point, which takes
its scratch from one static 128 MiB device array.  This file checks it,
through the C ABI, against the allocating gt_update_matrix on two calls in a
row (the shared array keeps the previous call's contents), checks that those
calls take no device memory from the library's pool (its live and pooled
bytes stay the same across them), and checks that an oversize refill and a
host-memory coefficient are refused.  The file sorts last so that a run
stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import gtgpu as GT
from gtgpu import _lib

pytestmark = pytest.mark.gpu

TOL = 1e-12    # same normwise FP64 tolerance as the other parity tests
TOL32 = 2e-6   # FP32 values: the two entry points may integrate in a different order


def _refill_noalloc(A, form, coef_dev, nu=0.3):
    lib = _lib.load()
    ptr = None if coef_dev is None else C.c_void_p(coef_dev.data_ptr())
    return lib.gt_update_matrix_noalloc(A.h, form, ptr, C.c_double(nu))


def _compare(A, B):
    _, _, va = A.csr()
    _, _, vb = B.csr()
    assert np.abs(va - vb).max() <= TOL * np.abs(va).max()


def test_noalloc_refill_matches_update_matrix_p1():
    torch = pytest.importorskip("torch")
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (12, 11, 10), simplexify=True)
    GT.jitter_interior_nodes(m, 0.2, 3)
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    k0 = GT.lognormal_cells(m.num_cells, 1.0, 1)
    A = GT.assemble_matrix(GT.laplacian(k0), np.float64, V, V)
    B = GT.assemble_matrix(GT.laplacian(k0), np.float64, V, V)
    ctx = B.ctx
    coefs = [torch.from_numpy(GT.lognormal_cells(m.num_cells, 1.0, seed)).cuda() for seed in (21, 22)]
    ctx.synchronize()
    for k in coefs:  # two calls in a row
        held = ctx.memory()  # (live, pooled) bytes of the library's pool
        st = _refill_noalloc(B, _lib.GT_LAPLACE, k)
        assert st == 0, ctx.lib.gt_last_error(ctx.h)
        assert ctx.memory() == held, "the refill took device memory from the pool"
        GT.update_matrix(A, GT.laplacian(k.cpu().numpy()))
        _compare(A, B)


def test_noalloc_refill_matches_update_matrix_q2_elasticity_fp32():
    torch = pytest.importorskip("torch")
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (4, 3, 3))
    V = GT.lagrange_space(GT.interior(m), 2, tensor_size=(3,), dirichlet_boundary=GT.boundary(m, ["2-face-5"]))
    A = GT.assemble_matrix(GT.elasticity(1.0, 0.3), np.float32, V, V)
    B = GT.assemble_matrix(GT.elasticity(1.0, 0.3), np.float32, V, V)
    for seed in (31, 32):
        E = GT.lognormal_cells(m.num_cells, 0.5, seed)
        GT.update_matrix(A, GT.elasticity(E, 0.3))
        assert _refill_noalloc(B, _lib.GT_ELASTICITY, torch.from_numpy(E).cuda()) == 0
        va, vb = A.values32().astype(np.float64), B.values32().astype(np.float64)
        assert np.abs(va - vb).max() <= TOL32 * np.abs(va).max()


def test_noalloc_refuses_oversize_and_host_memory():
    torch = pytest.importorskip("torch")
    # 2.06M cells x 10 packed entries x 8 B > 128 MiB
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (70, 70, 70), simplexify=True)
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    A = GT.assemble_matrix(GT.laplacian(), np.float64, V, V)
    assert _refill_noalloc(A, _lib.GT_LAPLACE, None) == _lib.GT_ERR_INVALID
    small = GT.cartesian_mesh((0, 1, 0, 1), (4, 4))
    W = GT.lagrange_space(GT.interior(small), 1)
    B = GT.assemble_matrix(GT.laplacian(), np.float64, W, W)
    host = np.ones(small.num_cells)
    st = _lib.load().gt_update_matrix_noalloc(B.h, _lib.GT_LAPLACE, C.c_void_p(host.ctypes.data), C.c_double(0.3))
    assert st == _lib.GT_ERR_INVALID
    # the matrix is unchanged and still refillable afterwards
    assert _refill_noalloc(B, _lib.GT_LAPLACE, torch.ones(small.num_cells, dtype=torch.float64, device="cuda")) == 0
