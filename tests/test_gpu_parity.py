"""GPU path (through the C ABI) against the CPU oracle on the same seeded
inputs: DOF ids and sparsity bit-exact, FP64 values within 1e-12 (normwise,
relative to the largest entry), FP32 values within 2e-6, vectors, solves."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

import gtgpu as GT
import oracle as O

pytestmark = pytest.mark.gpu

TOL64 = 1e-12   # plain FP64 path vs FP64 oracle
TOL32 = 2e-6    # FP32 element integration / values vs FP64 oracle


def _oracle_mesh(m):
    return dict(D=m.D, ctype=m.cell_type, coords=m.coords, cell_nodes=m.cell_nodes, pf0=m.corners,
                pf1=m.bedges if m.D == 3 else m.bfaces, pf1g=m.bface_group if m.D == 2 else None,
                pf2=m.bfaces if m.D == 3 else None, pf2g=m.bface_group if m.D == 3 else None,
                cells=m.cells_per_dir, box=m.domain)


def _oracle_space(m, order, ncomp, groups):
    om = _oracle_mesh(m)
    if m.D == 2:
        om["pf1"], om["pf1g"] = m.bfaces, m.bface_group
    return O.lagrange_space(om, order, ncomp=ncomp, dirichlet=groups), om


CASES = [
    # (id, cells, simplex, order, ncomp, dirichlet groups, form, jitter, coef sigma)
    ("q1quad_64x64", (64, 64), False, 1, 1, "boundary", O.LAPLACE, 0.0, 0.0),
    ("p1tet_6x5x4_jitter", (6, 5, 4), True, 1, 1, "boundary", O.LAPLACE, 0.2, 1.0),
    ("p1tet_4_mass", (4, 4, 4), True, 1, 1, None, O.MASS, 0.2, 0.5),
    ("q1hex_5x4x3_x0", (5, 4, 3), False, 1, 1, ["2-face-5"], O.LAPLACE, 0.15, 1.0),
    ("q1hex_elast", (4, 3, 3), False, 1, 3, ["2-face-5"], O.ELASTICITY, 0.1, 0.5),
    ("q2quad_5x7", (5, 7), False, 2, 1, "boundary", O.LAPLACE, 0.2, 1.0),
    ("q2quad_mass_vec", (3, 4), False, 2, 2, ["1-face-1", "1-face-3"], O.MASS, 0.0, 0.0),
    ("q2hex_elast_x0", (3, 4, 5), False, 2, 3, ["2-face-5"], O.ELASTICITY, 0.1, 0.5),
    ("q2hex_lap_free", (3, 3, 3), False, 2, 1, None, O.LAPLACE, 0.0, 0.0),
    ("q2hex_elast_affine", (3, 3, 4), False, 2, 3, ["2-face-5"], O.ELASTICITY, 0.0, 0.5),
    ("q1hex_lap_affine", (4, 5, 3), False, 1, 1, "boundary", O.LAPLACE, 0.0, 1.0),
    ("q2quad_veclap_affine", (4, 3), False, 2, 2, ["1-face-3"], O.LAPLACE, 0.0, 1.0),
    ("q1quad_elast_affine", (5, 4), False, 1, 2, ["1-face-3"], O.ELASTICITY, 0.0, 0.5),
    ("q1quad_1x1_alldiri", (1, 1), False, 1, 1, "boundary", O.LAPLACE, 0.0, 0.0),
    ("q2quad_1x1", (1, 1), False, 2, 1, "boundary", O.LAPLACE, 0.0, 0.0),
    ("p2tet_3x2x2_jitter", (3, 2, 2), True, 2, 1, "boundary", O.LAPLACE, 0.2, 1.0),
    ("p2tet_mass_free", (2, 2, 2), True, 2, 1, None, O.MASS, 0.1, 0.5),
    ("p2tet_elast_x0", (2, 2, 3), True, 2, 3, ["2-face-5"], O.ELASTICITY, 0.1, 0.5),
    ("p2tet_1x1x1", (1, 1, 1), True, 2, 1, "boundary", O.LAPLACE, 0.0, 0.0),
]

_KIND = {O.LAPLACE: GT.laplacian, O.MASS: GT.mass, O.ELASTICITY: GT.elasticity}


def _build(case):
    cid, cells, simplex, order, ncomp, groups, form, jit, sig = case
    D = len(cells)
    m = GT.cartesian_mesh(tuple(x for _ in cells for x in (0.0, 1.0)), cells, simplexify=simplex)
    if jit:
        GT.jitter_interior_nodes(m, jit, 7)
    coef = GT.lognormal_cells(m.num_cells, sig, 11) if sig else None
    Om = GT.interior(m)
    diri = None if groups is None else GT.boundary(m, None if groups == "boundary" else groups)
    V = GT.lagrange_space(Om, order, tensor_size=(ncomp,) if ncomp > 1 else None, dirichlet_boundary=diri)
    ref, om = _oracle_space(m, order, ncomp, None if groups is None else groups)
    a = _KIND[form](coef) if form != O.ELASTICITY else GT.elasticity(coef, 0.3)
    return m, V, ref, a, coef, form, order


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_dof_numbering_bit_exact(case):
    m, V, ref, *_ = _build(case)
    assert V.num_free_dofs == ref["nfree"] and V.num_dirichlet_dofs == ref["ndiri"]
    assert np.array_equal(V.face_dofs(), ref["cell_dofs"])


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_matrix_pattern_and_fp64_values(case):
    m, V, ref, a, coef, form, order = _build(case)
    A = GT.assemble_matrix(a, np.float64, V, V)
    rp, ci, v = A.csr()
    cp, rv, nz = O.assemble_matrix(ref, form, 2 * order, coef=coef, nu=0.3)
    orp, oci, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    if ov.size:
        scale = np.abs(ov).max()
        assert np.abs(v - ov).max() <= TOL64 * scale


_FP32_CASES = CASES[:8] + [c for c in CASES if c[0] == "p2tet_3x2x2_jitter"]


@pytest.mark.parametrize("case", _FP32_CASES, ids=[c[0] for c in _FP32_CASES])
def test_fp32_and_mixed_values(case):
    m, V, ref, a, coef, form, order = _build(case)
    cp, rv, nz = O.assemble_matrix(ref, form, 2 * order, coef=coef, nu=0.3)
    _, _, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    A32 = GT.assemble_matrix(a, np.float32, V, V)
    v32 = A32.values32()
    scale = np.abs(ov).max()
    assert np.abs(v32 - ov).max() <= TOL32 * scale
    Am = GT.assemble_matrix(a, "mixed", V, V)
    _, _, v64 = Am.csr()
    # mixed: FP64-integrated FP64 values, FP32-integrated FP32 values (the
    # same FP32 pass as the FP32 assembly)
    assert np.abs(v64 - ov).max() <= TOL64 * scale
    assert np.array_equal(Am.values32(), v32)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_vector(case):
    m, V, ref, a, coef, form, order = _build(case)
    ncomp = V.ncomp
    f = np.array([0.0, 0.0, -1.0])[-ncomp:] if ncomp > 1 else 1.0
    b = GT.assemble_vector(GT.source(f, coef), np.float64, V)
    ob = O.assemble_vector(ref, 2 * order, f, coef=coef)
    if ob.size:
        assert np.abs(b - ob).max() <= TOL64 * np.abs(ob).max()
    # combined entry point: the same vector (its affine-cell path factorises
    # the quadrature sum, so agreement is to rounding, not bitwise)
    A2, b2 = GT.assemble_matrix_and_vector(a, GT.source(f, coef), np.float64, V)
    if ob.size:
        assert np.abs(b2 - ob).max() <= TOL64 * np.abs(ob).max()


def test_assembly_is_deterministic():
    m, V, ref, a, coef, form, order = _build(CASES[1])
    A1 = GT.assemble_matrix(a, np.float64, V, V)
    A2 = GT.assemble_matrix(a, np.float64, V, V)
    assert np.array_equal(A1.csr()[2], A2.csr()[2])


@pytest.mark.parametrize("ci", [1, 3, 15])
def test_fused_load_vector_is_bitwise_the_separate_pass(ci):
    # P1 tets (packed element matrices), non-affine Q1 hexes, P2 tets: the
    # element vectors come from the same kernel either way, and the fused
    # scatter sums them in the order of the separate vector pass
    m, V, ref, a, coef, form, order = _build(CASES[ci])
    l = GT.source(1.0, coef)
    b1 = GT.assemble_vector(l, np.float64, V)
    _, b2 = GT.assemble_matrix_and_vector(a, l, np.float64, V)
    assert np.array_equal(b1, b2)


def test_update_matrix_equals_fresh_assembly():
    m, V, ref, a, coef, form, order = _build(CASES[1])
    A = GT.assemble_matrix(a, np.float64, V, V)
    k2 = GT.lognormal_cells(m.num_cells, 1.0, 99)
    GT.update_matrix(A, GT.laplacian(k2))
    B = GT.assemble_matrix(GT.laplacian(k2), np.float64, V, V)
    assert np.array_equal(A.csr()[2], B.csr()[2])


def test_unsupported_forms_raise():
    m = GT.cartesian_mesh((0, 1, 0, 1), (4, 4))
    V = GT.lagrange_space(GT.interior(m), 1)
    with pytest.raises(NotImplementedError):
        GT.assemble_matrix(lambda u, v: None, np.float64, V, V)
    with pytest.raises(GT.GTError):
        GT.assemble_matrix(GT.elasticity(None, 0.3), np.float64, V, V)  # scalar space


@pytest.mark.parametrize("mode", ["fp64", "ir"])
def test_solve_cfg1_poisson(mode):
    """2-D Poisson -lap u = 1, 64x64 Q1, CG to 1e-10 (plain) / IR to 1e-10."""
    m = GT.cartesian_mesh((0, 1, 0, 1), (64, 64))
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    T = np.float64 if mode == "fp64" else "mixed"
    A, b = GT.assemble_matrix_and_vector(GT.laplacian(), GT.source(1.0), T, V)
    x, info = GT.solve(A, b, rtol=1e-10, mode=mode)
    assert info["converged"] and info["rel_residual"] <= 1e-10
    ref, _ = _oracle_space(m, 1, 1, "boundary")
    cp, rv, nz = O.assemble_matrix(ref, O.LAPLACE, 2)
    xd = sla.spsolve(sp.csc_matrix((nz, rv, cp), shape=(ref["nfree"],) * 2), O.assemble_vector(ref, 2, 1.0))
    assert np.abs(x - xd).max() / np.abs(xd).max() < 1e-8


@pytest.mark.parametrize("mode", ["fp64", "ir"])
def test_large_solve_replays_captured_cg_chunks(mode):
    """72^3 x 6 P1 tets (357,911 free rows): above the single persistent
    kernel's range, so the CG runs as one launch per phase, each chunk of
    iterations replayed from a captured CUDA graph; converged on the FP64
    true residual and equal to a sparse direct solve."""
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (72, 72, 72), simplexify=True)
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    T = np.float64 if mode == "fp64" else "mixed"
    A, b = GT.assemble_matrix_and_vector(GT.laplacian(), GT.source(1.0), T, V)
    assert A.shape[0] > 262144
    g0 = V.ctx.graph_launches()
    x, info = GT.solve(A, b, rtol=1e-9, mode=mode)
    assert info["converged"] and info["rel_residual"] <= 1e-9
    assert V.ctx.graph_launches() > g0
    r = b - A.tocsr() @ x
    assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(b) * 1.01


def test_solve_q2_elasticity_ir():
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (4, 4, 4))
    V = GT.lagrange_space(GT.interior(m), 2, tensor_size=(3,), dirichlet_boundary=GT.boundary(m, ["2-face-5"]))
    A, b = GT.assemble_matrix_and_vector(GT.elasticity(1.0, 0.3), GT.source([0, 0, -1.0]), "mixed", V)
    x, info = GT.solve(A, b, rtol=1e-10, mode="ir")
    assert info["converged"]
    xd = sla.spsolve(A.tocsr().tocsc(), b)
    assert np.abs(x - xd).max() / np.abs(xd).max() < 1e-8


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_spmv_matches_csr(case):
    """gt_spmv (the sliced-ELL copy for scalar matrices, the block-CSR kernel
    otherwise) against the downloaded CSR times the same vector on the host."""
    m, V, ref, a, coef, form, order = _build(case)
    A = GT.assemble_matrix(a, np.float64, V, V)
    n = A.shape[0]
    if n == 0:
        return
    x = np.random.default_rng(5).standard_normal(n)
    y = A @ x
    yr = A.tocsr() @ x
    assert np.abs(y - yr).max() <= 1e-13 * max(1.0, np.abs(yr).max())


def test_spmv_copy_follows_value_updates():
    """the SpMV's cached copy is refilled after update_matrix: a product after
    the update equals the product with the updated CSR, not the first one"""
    m, V, ref, a, coef, form, order = _build(CASES[1])
    A = GT.assemble_matrix(a, np.float64, V, V)
    x = np.random.default_rng(6).standard_normal(A.shape[0])
    y1 = A @ x  # builds the copy
    k2 = GT.lognormal_cells(m.num_cells, 1.0, 99)
    GT.update_matrix(A, GT.laplacian(k2))
    y2 = A @ x
    yr = A.tocsr() @ x
    assert np.abs(y2 - yr).max() <= 1e-13 * np.abs(yr).max()
    assert np.abs(y2 - y1).max() > 1e-6 * np.abs(yr).max()
    # a solve after the update uses the refreshed copy as well
    b = np.ones(A.shape[0])
    xs, info = GT.solve(A, b, rtol=1e-10, mode="fp64")
    assert info["converged"]
    assert np.abs(A.tocsr() @ xs - b).max() <= 1e-8 * np.abs(b).max()


def _fan_mesh(n):
    """A double pyramid over an n-gon: 2n tetrahedra around one centre node,
    whose incidence list (2n cells) is longer than the row-per-thread
    sparsity pass holds -- the warp kernel recounts."""
    from gtgpu.mesh import Mesh
    t = np.linspace(0.0, 2.0 * np.pi, n, endpoint=False)
    ring = np.column_stack([np.cos(t), np.sin(t), np.zeros(n)])
    coords = np.vstack([[0.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.0, 0.0, -1.0], ring])
    cells, faces = [], []
    for i in range(n):
        a, b = 4 + i, 4 + (i + 1) % n  # 1-based ring nodes
        cells += [[1, a, b, 2], [1, a, b, 3]]
        faces += [[a, b, 2], [a, b, 3]]
    faces = np.asarray(faces, np.int32)
    return Mesh(D=3, cell_type=GT.api._lib.GT_TET4, coords=coords, cell_nodes=np.asarray(cells, np.int32),
                corners=np.zeros(0, np.int32), bfaces=faces, bface_group=np.ones(len(faces), np.int32),
                bedges=np.zeros((0, 2), np.int32))


@pytest.mark.parametrize("dirichlet", [False, True])
def test_pattern_rows_beyond_the_thread_pass(dirichlet):
    m = _fan_mesh(20)  # 40 cells around node 1
    diri = GT.boundary(m) if dirichlet else None
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=diri)
    A = GT.assemble_matrix(GT.laplacian(), np.float64, V, V)
    rp, ci, v = A.csr()
    om = dict(D=3, ctype=m.cell_type, coords=m.coords, cell_nodes=m.cell_nodes, pf0=m.corners, pf1=m.bedges,
              pf1g=None, pf2=m.bfaces, pf2g=m.bface_group, cells=(), box=())
    ref = O.lagrange_space(om, 1, dirichlet="boundary" if dirichlet else None)
    assert np.array_equal(V.face_dofs(), ref["cell_dofs"])
    cp, rv, nz = O.assemble_matrix(ref, O.LAPLACE, 2)
    orp, oci, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert np.abs(v - ov).max() <= TOL64 * np.abs(ov).max()


@pytest.mark.parametrize("n", [12, 20, 40])
def test_p1_scatter_row_lengths(n):
    """The centre row of a fan over an n-gon holds n + 3 columns: 15 (the
    scatter's 16-column slots), 23 (32-column slots) and 43 (the search over
    the row's length) -- FP64, FP32 values and the load vector against the
    oracle"""
    m = _fan_mesh(n)
    V = GT.lagrange_space(GT.interior(m), 1)
    coef = GT.lognormal_cells(m.num_cells, 0.5, 7)
    a = GT.laplacian(coef)
    A, b = GT.assemble_matrix_and_vector(a, GT.source(1.0, coef), np.float64, V)
    rp, ci, v = A.csr()
    assert np.diff(rp).max() == n + 3
    om = dict(D=3, ctype=m.cell_type, coords=m.coords, cell_nodes=m.cell_nodes, pf0=m.corners, pf1=m.bedges,
              pf1g=None, pf2=m.bfaces, pf2g=m.bface_group, cells=(), box=())
    ref = O.lagrange_space(om, 1)
    cp, rv, nz = O.assemble_matrix(ref, O.LAPLACE, 2, coef=coef)
    orp, oci, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert np.abs(v - ov).max() <= TOL64 * np.abs(ov).max()
    ob = O.assemble_vector(ref, 2, 1.0, coef=coef)
    assert np.abs(b - ob).max() <= TOL64 * np.abs(ob).max()
    v32 = GT.assemble_matrix(a, np.float32, V).values32()
    assert np.abs(v32 - ov).max() <= TOL32 * np.abs(ov).max()


def test_pattern_rows_wide_dof_spread():
    """Two layers of 180 x 180 cubes: the DOFs of a cell lie up to 181^2 + 182
    apart, beyond the count pass's 16-bit column offsets (it keeps 32-bit
    column ids there) -- pattern and values against the oracle"""
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 0.02), (180, 180, 2), simplexify=True)
    V = GT.lagrange_space(GT.interior(m), 1)
    cd = V.face_dofs()
    assert (cd.max(axis=1) - cd.min(axis=1)).max() >= 32768
    A = GT.assemble_matrix(GT.laplacian(), np.float64, V, V)
    rp, ci, v = A.csr()
    ref, om = _oracle_space(m, 1, 1, None)
    cp, rv, nz = O.assemble_matrix(ref, O.LAPLACE, 2)
    orp, oci, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert np.abs(v - ov).max() <= TOL64 * np.abs(ov).max()


def _graded(cells, order, ncomp, groups, form, sig):
    """A Cartesian mesh with x -> x^2 (and y -> y^1.5): every cell stays an
    axis-aligned box (affine), but cell sizes differ, so the sum-factorised
    path uses per-cell geometry records instead of one shared record."""
    D = len(cells)
    m = GT.cartesian_mesh(tuple(x for _ in cells for x in (0.0, 1.0)), cells)
    m.coords[:, 0] = m.coords[:, 0] ** 2
    m.coords[:, 1] = m.coords[:, 1] ** 1.5
    coef = GT.lognormal_cells(m.num_cells, sig, 11) if sig else None
    diri = None if groups is None else GT.boundary(m, None if groups == "boundary" else groups)
    V = GT.lagrange_space(GT.interior(m), order, tensor_size=(ncomp,) if ncomp > 1 else None, dirichlet_boundary=diri)
    ref, om = _oracle_space(m, order, ncomp, groups)
    a = _KIND[form](coef) if form != O.ELASTICITY else GT.elasticity(coef, 0.3)
    return m, V, ref, a, coef


GRADED = [((5, 4), 2, 1, "boundary", O.LAPLACE, 1.0), ((3, 4, 3), 2, 3, ["2-face-5"], O.ELASTICITY, 0.5),
          ((4, 3, 3), 1, 1, "boundary", O.MASS, 0.5), ((4, 5), 1, 2, ["1-face-3"], O.ELASTICITY, 0.0)]


@pytest.mark.parametrize("case", GRADED, ids=lambda c: f"{len(c[0])}d_q{c[1]}_bs{c[2]}_f{c[4]}")
def test_graded_affine_mesh(case):
    """affine, non-uniform cells: FP64, FP32 and mixed values and the load
    vector against the oracle"""
    cells, order, ncomp, groups, form, sig = case
    m, V, ref, a, coef = _graded(cells, order, ncomp, groups, form, sig)
    assert np.array_equal(V.face_dofs(), ref["cell_dofs"])
    cp, rv, nz = O.assemble_matrix(ref, form, 2 * order, coef=coef, nu=0.3)
    orp, oci, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    f = np.array([0.0, 0.0, -1.0])[-ncomp:] if ncomp > 1 else 1.0
    A, b = GT.assemble_matrix_and_vector(a, GT.source(f, coef), np.float64, V)
    rp, ci, v = A.csr()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    scale = np.abs(ov).max()
    assert np.abs(v - ov).max() <= TOL64 * scale
    ob = O.assemble_vector(ref, 2 * order, f, coef=coef)
    assert np.abs(b - ob).max() <= TOL64 * np.abs(ob).max()
    v32 = GT.assemble_matrix(a, np.float32, V).values32()
    assert np.abs(v32 - ov).max() <= TOL32 * scale
    Am = GT.assemble_matrix(a, "mixed", V)
    assert np.abs(Am.csr()[2] - ov).max() <= TOL64 * scale
    assert np.array_equal(Am.values32(), v32)


_AFFINE = [c for c in CASES if c[7] == 0.0 and not c[2] and c[1] != (1, 1)]


@pytest.mark.parametrize("case", _AFFINE, ids=[c[0] for c in _AFFINE])
def test_uniform_geometry_path_matches_per_cell_records(case, monkeypatch):
    """Uniform Cartesian meshes take the shared-record path (one reference
    block scaled per cell); a context created with GTGPU_UNIFORM=0 takes the
    per-cell records.  Both agree with each other and with the oracle."""
    m, V, ref, a, coef, form, order = _build(case)
    A = GT.assemble_matrix(a, np.float64, V, V)
    monkeypatch.setenv("GTGPU_UNIFORM", "0")
    ctx2 = GT.Context(0)
    monkeypatch.delenv("GTGPU_UNIFORM")
    V2 = GT.lagrange_space(GT.interior(m), order, tensor_size=(V.ncomp,) if V.ncomp > 1 else None,
                           dirichlet_boundary=None if case[5] is None else
                           GT.boundary(m, None if case[5] == "boundary" else case[5]), ctx=ctx2)
    B = GT.assemble_matrix(a, np.float64, V2, V2)
    _, _, va = A.csr()
    _, _, vb = B.csr()
    cp, rv, nz = O.assemble_matrix(ref, form, 2 * order, coef=coef, nu=0.3)
    _, _, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    if ov.size:
        scale = np.abs(ov).max()
        assert np.abs(va - ov).max() <= TOL64 * scale and np.abs(vb - ov).max() <= TOL64 * scale
        assert np.abs(va - vb).max() <= 1e-13 * scale
    del B, V2
    m._device.pop(id(ctx2), None)
    ctx2.close()


@pytest.mark.parametrize("form", [O.LAPLACE, O.MASS])
def test_p1_double_float_kernel_matches_fp64_kernel(form, monkeypatch):
    """FP64-valued P1 element matrices are computed in double-float (pairs of
    FP32) by default; a context created with GTGPU_P1=fp64 takes the FP64
    kernel.  Matrices and load vectors agree with each other to 1e-13 and
    with the oracle to 1e-12 (of the largest entry)."""
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (20, 18, 16), simplexify=True)
    GT.jitter_interior_nodes(m, 0.2, 31)
    kappa = GT.lognormal_cells(m.num_cells, 1.0, 32)
    a = GT.laplacian(kappa) if form == O.LAPLACE else GT.mass(kappa)
    l = GT.source(1.0, kappa)
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    A, b = GT.assemble_matrix_and_vector(a, l, np.float64, V)
    monkeypatch.setenv("GTGPU_P1", "fp64")
    ctx2 = GT.Context(0)
    monkeypatch.delenv("GTGPU_P1")
    V2 = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m), ctx=ctx2)
    A2, b2 = GT.assemble_matrix_and_vector(a, l, np.float64, V2)
    _, _, v = A.csr()
    _, _, v2 = A2.csr()
    scale = np.abs(v2).max()
    assert np.abs(v - v2).max() <= 1e-13 * scale
    assert np.abs(b - b2).max() <= 1e-13 * np.abs(b2).max()
    ref, _ = _oracle_space(m, 1, 1, "boundary")
    cp, rv, nz = O.assemble_matrix(ref, form, 2, coef=kappa)
    _, _, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    assert np.abs(v - ov).max() <= TOL64 * np.abs(ov).max()
    ob = O.assemble_vector(ref, 2, 1.0, coef=kappa)
    assert np.abs(b - ob).max() <= TOL64 * np.abs(ob).max()
    del A2, V2
    m._device.pop(id(ctx2), None)
    ctx2.close()
