"""Failure statuses of the C ABI, each made to happen without faulting or
hanging the GPU, and the context still working afterwards:

  GT_ERR_NOT_CONVERGED  a solve that reaches maxit (single and batched)
  GT_ERR_INVALID        a malformed mesh: a node id out of range, a cell with
                        det J = 0
  GT_ERR_TIMEOUT        the persistent solver's grid barrier waiting for an
                        arrival that never comes, given up after its limit

An inverted cell (det J < 0) is not an error: the reference integrates with
|det J| (change_of_measure, src/quadrature.jl:4-6), and so does this path."""
import ctypes as C

import numpy as np
import pytest

import gtgpu as GT
from gtgpu import _lib
from gtgpu import batch as GB

pytestmark = pytest.mark.gpu


def _poisson(n=6):
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (n, n, n), simplexify=True)
    GT.jitter_interior_nodes(m, 0.2, 3)
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    A, b = GT.assemble_matrix_and_vector(GT.laplacian(GT.lognormal_cells(m.num_cells, 1.0, 3)), GT.source(1.0),
                                         "mixed", V)
    return m, V, A, b


@pytest.mark.parametrize("mode", ["fp64", "ir"])
def test_not_converged_at_maxit(mode):
    m, V, A, b = _poisson()
    x, info = GT.solve(A, b, rtol=1e-12, maxit=3, mode=mode, raise_on_fail=False)
    assert not info["converged"] and info["iterations"] <= 3 and info["rel_residual"] > 1e-12
    with pytest.raises(GT.GTError) as e:
        GT.solve(A, b, rtol=1e-12, maxit=3, mode=mode)
    assert e.value.code == _lib.GT_ERR_NOT_CONVERGED
    x, info = GT.solve(A, b, rtol=1e-10, mode=mode)  # the context still solves
    assert info["converged"] and info["rel_residual"] <= 1e-10


def test_batch_not_converged_at_maxit():
    inst = [GB.assemble_instance(s, seed=5, T="mixed") for s in
            (GB.InstanceSpec(0, 2, 1, 12), GB.InstanceSpec(1, 3, 2, 3))]
    B = GB.Batch([A for _, _, A, _ in inst])
    bs = [b for _, _, _, b in inst]
    with pytest.raises(GT.GTError) as e:
        B.solve(bs, rtol=1e-12, maxit=2, mode="ir")
    assert e.value.code == _lib.GT_ERR_NOT_CONVERGED
    x, infos = B.solve(bs, rtol=1e-12, maxit=2, mode="ir", raise_on_fail=False)
    assert all(i["rel_residual"] > 1e-12 for i in infos)
    x, infos = B.solve(bs, rtol=1e-10, mode="ir")
    assert all(i["rel_residual"] <= 1e-10 for i in infos)


@pytest.mark.parametrize("bad", ["past_the_end", "zero"])
def test_node_id_out_of_range(bad):
    m = GT.cartesian_mesh((0, 1, 0, 1), (3, 3))
    m.cell_nodes[4, 2] = m.num_nodes + 7 if bad == "past_the_end" else 0  # ids are 1-based
    with pytest.raises(GT.GTError) as e:
        GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    assert e.value.code == _lib.GT_ERR_INVALID and "out of range" in str(e.value)
    m2 = GT.cartesian_mesh((0, 1, 0, 1), (3, 3))  # a valid mesh still works
    V = GT.lagrange_space(GT.interior(m2), 1, dirichlet_boundary=GT.boundary(m2))
    assert V.num_free_dofs == 4


@pytest.mark.parametrize("precision", [np.float64, np.float32])
def test_degenerate_cell(precision):
    # the interior node (1,1,1) of a 2x2x2 tet mesh moved onto its neighbour
    # (0,1,1): the tets holding the edge between them have two coincident
    # vertices, so det J = 0 exactly
    m = GT.cartesian_mesh((0, 2, 0, 2, 0, 2), (2, 2, 2), simplexify=True)
    good = m.coords.copy()
    centre, left = 1 + 3 + 9, 0 + 3 + 9  # x-fastest node numbering, 0-based
    m.coords[centre] = m.coords[left]
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    with pytest.raises(GT.GTError) as e:
        GT.assemble_matrix(GT.laplacian(), precision, V)
    assert e.value.code == _lib.GT_ERR_INVALID and "degenerate" in str(e.value)
    V.dmesh.set_coords(good)  # repaired coordinates: the same space assembles
    A = GT.assemble_matrix(GT.laplacian(), precision, V)
    assert A.nnz == 1


def test_inverted_cells_integrate_with_abs_det():
    import oracle as O
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (3, 2, 2))
    GT.jitter_interior_nodes(m, 0.15, 8)
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m, ["2-face-5"]))
    A = GT.assemble_matrix(GT.laplacian(), np.float64, V)
    mirrored = m.coords.copy()
    mirrored[:, 0] = 1.0 - mirrored[:, 0]  # every cell inverted: det J < 0
    V.dmesh.set_coords(mirrored)
    Am = GT.assemble_matrix(GT.laplacian(), np.float64, V)
    _, _, v = A.csr()
    _, _, vm = Am.csr()
    assert np.abs(vm - v).max() <= 1e-12 * np.abs(v).max()
    om = dict(D=3, ctype=O.HEX8, coords=mirrored, cell_nodes=m.cell_nodes, pf0=m.corners, pf1=m.bedges,
              pf2=m.bfaces, pf2g=m.bface_group)
    ref = O.lagrange_space(om, 1, dirichlet=["2-face-5"])
    cp, rv, nz = O.assemble_matrix(ref, O.LAPLACE, 2)
    _, _, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    assert np.abs(vm - ov).max() <= 1e-12 * np.abs(ov).max()


def test_grid_barrier_times_out():
    ctx = GT.default_context()
    lib = ctx.lib
    assert lib.gt_ctx_barrier_probe(ctx.h, 16, 0, 200_000_000) == _lib.GT_OK
    st = lib.gt_ctx_barrier_probe(ctx.h, 16, 1, 50_000_000)  # one arrival never comes
    assert st == _lib.GT_ERR_TIMEOUT
    assert b"timed out" in lib.gt_last_error(ctx.h)
    assert lib.gt_ctx_barrier_probe(ctx.h, 0, 0, 1000) == _lib.GT_ERR_INVALID
    # the context still runs the persistent solver afterwards
    m, V, A, b = _poisson(4)
    x, info = GT.solve(A, b, rtol=1e-10, mode="fp64")
    assert info["converged"]
    n = C.c_int64()
    assert lib.gt_ctx_launch_count(ctx.h, C.byref(n)) == 0 and n.value > 0


@pytest.mark.parametrize("n", [6, 20, 72])
def test_unattainable_tolerance_stops_without_diverging(n):
    """A tolerance below FP64's attainable accuracy: the CG (persistent kernel
    for the small system, one launch per phase for the 357k-row one) ends as
    not converged after a few true-residual checks without progress, with
    the residual at the attainable level -- it neither runs to maxit nor
    diverges (the directions restart when the recurrence has drifted from
    the true residual)."""
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (n, n, n), simplexify=True)
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    A, b = GT.assemble_matrix_and_vector(GT.laplacian(), GT.source(1.0), "mixed", V)
    _, ok = GT.solve(A, b, rtol=1e-10, mode="fp64")
    for mode in ("fp64", "ir"):
        for rtol in (1e-14, 1e-19):  # at and below the attainable accuracy
            x, info = GT.solve(A, b, rtol=rtol, maxit=200000, mode=mode, raise_on_fail=False)
            assert info["iterations"] < 20 * ok["iterations"] + 400, (mode, rtol, info)
            assert info["rel_residual"] < 1e-12, (mode, rtol, info)
            assert info["converged"] or rtol == 1e-19 or info["rel_residual"] > rtol
    B = GB.Batch([A]) if n == 6 else None
    if B is not None:
        xb, infos = B.solve([b], rtol=1e-19, maxit=200000, mode="fp64", raise_on_fail=False)
        assert infos[0]["iterations"] < 20 * ok["iterations"] + 200 and infos[0]["rel_residual"] < 1e-12
