"""Boundary integrals int g v dGamma (gt_assemble_boundary_vector, the
Neumann term) on the GPU: partition of unity (sum of the vector = g |Gamma|),
the integral of a linear function through the nodal values, Neumann patch
tests solved to round-off, and determinism."""
import numpy as np
import pytest

import gtgpu as GT

pytestmark = pytest.mark.gpu

CASES = [
    # (id, box cells, simplex, order, jitter)
    ("p1tet", (4, 3, 5), True, 1, 0.2),
    ("p2tet", (2, 3, 2), True, 2, 0.2),
    ("q1hex", (3, 4, 2), False, 1, 0.15),
    ("q2hex", (2, 3, 2), False, 2, 0.1),
    ("q1quad", (5, 4), False, 1, 0.2),
    ("q2quad", (3, 2), False, 2, 0.0),
]


def _mesh(cells, simplex, jit):
    m = GT.cartesian_mesh(tuple(x for _ in cells for x in (0.0, 1.0)), cells, simplexify=simplex)
    if jit:
        GT.jitter_interior_nodes(m, jit, 4)  # boundary nodes stay: the box faces stay planar
    return m


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_partition_of_unity_and_linear_moments(case):
    cid, cells, simplex, order, jit = case
    m = _mesh(cells, simplex, jit)
    D = len(cells)
    V = GT.lagrange_space(GT.interior(m), order)  # no Dirichlet: every node free
    g = 1.75
    top = f"{D - 1}-face-{2 * D}"  # x = 1
    b_all = GT.assemble_boundary_vector(g, GT.boundary(m), V)
    b_x1 = GT.assemble_boundary_vector(g, GT.boundary(m, [top]), V)
    assert abs(b_all.sum() - g * 2 * D) < 1e-12
    assert abs(b_x1.sum() - g) < 1e-12
    xf, _ = V.node_coordinates()
    # int_{x=1} g y dGamma = g / 2 ; int_{all} g x dGamma = g * (2 D - 1) / 2 ... computed per face:
    # faces x=0 and x=1 give 0 and 1, the 2(D-1) others give 1/2 each
    assert abs(b_x1 @ xf[:, 1] - g / 2) < 1e-12
    assert abs(b_all @ xf[:, 0] - g * (1 + (2 * D - 2) / 2)) < 1e-12
    # accumulation adds
    b2 = GT.assemble_boundary_vector(g, GT.boundary(m, [top]), V, out=b_all.copy(), accumulate=True)
    assert np.allclose(b2, b_all + b_x1, rtol=0, atol=1e-14)
    # bitwise reproducible
    assert np.array_equal(GT.assemble_boundary_vector(g, GT.boundary(m), V), b_all)


def test_neumann_patch_tests():
    # P1 tets: u = 1 + x + 2y + 3z, Neumann du/dn = 1 on x = 1, Dirichlet elsewhere
    m = _mesh((4, 4, 3), True, 0.2)
    diri = GT.boundary(m, [f"2-face-{k}" for k in (1, 2, 3, 4, 5)])
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=diri)
    p = GT.Polynomial(c0=1.0, x=1.0, y=2.0, z=3.0)
    xd = GT.interpolate_dirichlet(p, V)
    lp = GT.linear_problem(V, GT.laplacian(), GT.source(0.0), dirichlet_values=xd,
                           neumann=[(1.0, GT.boundary(m, ["2-face-6"]))])
    x, _ = GT.solve(lp, rtol=1e-13)
    assert GT.l2_error(V, x, p, xd) < 1e-10
    # Q2 hexes: u = x^2 + y, -lap u = -2, du/dn = 2 on x = 1
    m2 = _mesh((3, 2, 2), False, 0.0)
    diri2 = GT.boundary(m2, [f"2-face-{k}" for k in (1, 2, 3, 4, 5)])
    V2 = GT.lagrange_space(GT.interior(m2), 2, dirichlet_boundary=diri2)
    q = GT.Polynomial(y=1.0, xx=1.0)
    xd2 = GT.interpolate_dirichlet(q, V2)
    lp2 = GT.linear_problem(V2, GT.laplacian(), GT.source(-2.0), dirichlet_values=xd2,
                            neumann=[(2.0, GT.boundary(m2, ["2-face-6"]))])
    x2, _ = GT.solve(lp2, rtol=1e-13)
    assert GT.l2_error(V2, x2, q, xd2) < 1e-10 and GT.h1_error(V2, x2, q, xd2) < 1e-9
    # Q1 quads: u = x - y, du/dn = 1 on x = 1 (1-face-4)
    m3 = _mesh((6, 5), False, 0.2)
    V3 = GT.lagrange_space(GT.interior(m3), 1, dirichlet_boundary=GT.boundary(m3, ["1-face-1", "1-face-2", "1-face-3"]))
    r = GT.Polynomial(x=1.0, y=-1.0)
    xd3 = GT.interpolate_dirichlet(r, V3)
    lp3 = GT.linear_problem(V3, GT.laplacian(), GT.source(0.0), dirichlet_values=xd3,
                            neumann=[(1.0, GT.boundary(m3, ["1-face-4"]))])
    x3, _ = GT.solve(lp3, rtol=1e-13)
    assert GT.l2_error(V3, x3, r, xd3) < 1e-10


def test_vector_traction():
    m = _mesh((2, 2, 2), False, 0.0)
    V = GT.lagrange_space(GT.interior(m), 2, tensor_size=(3,))
    g = np.array([0.5, -1.0, 2.0])
    b = GT.assemble_boundary_vector(g, GT.boundary(m, ["2-face-2"]), V)  # z = 1, area 1
    assert np.allclose(b.reshape(-1, 3).sum(axis=0), g, rtol=0, atol=1e-12)


def _oracle_space(m, order, ncomp, groups):
    import oracle as O
    om = dict(D=m.D, ctype=m.cell_type, coords=m.coords, cell_nodes=m.cell_nodes, pf0=m.corners,
              cells=m.cells_per_dir, box=m.domain)
    if m.D == 2:
        om["pf1"], om["pf1g"] = m.bfaces, m.bface_group
    else:
        om["pf1"], om["pf2"], om["pf2g"] = m.bedges, m.bfaces, m.bface_group
    return O.lagrange_space(om, order, ncomp=ncomp, dirichlet=groups)


ORACLE_CASES = [
    # (id, cells, simplex, order, ncomp, jitter, Dirichlet groups, Neumann groups, g)
    ("p1tet_x1", (4, 3, 5), True, 1, 1, 0.2, ["2-face-1", "2-face-2"], ["2-face-6"], 1.0),
    ("p1tet_sides", (4, 3, 5), True, 1, 1, 0.2, ["2-face-5"], ["2-face-6", "2-face-1"], -0.75),
    ("p2tet_all", (2, 3, 2), True, 2, 1, 0.2, None, None, 1.5),
    ("q1hex_z1", (3, 4, 2), False, 1, 1, 0.15, ["2-face-5"], ["2-face-2"], 2.0),
    ("q2hex_vec", (2, 3, 2), False, 2, 3, 0.1, ["2-face-5"], ["2-face-6", "2-face-3"], [0.5, -1.0, 2.0]),
    ("q1quad_all", (5, 4), False, 1, 1, 0.2, ["1-face-3"], None, 1.25),
    ("q2quad_vec", (3, 2), False, 2, 2, 0.0, ["1-face-1"], ["1-face-4"], [1.0, -2.0]),
]


@pytest.mark.parametrize("case", ORACLE_CASES, ids=[c[0] for c in ORACLE_CASES])
def test_boundary_vector_matches_oracle(case):
    """gt_assemble_boundary_vector entry by entry against the oracle's
    restatement of assemble_in_Γn! (same faces, same free DOFs; the two sum
    each DOF's faces in different orders and use different exact triangle
    rules, so they agree to rounding: 1e-12 of the largest entry)."""
    import oracle as O
    cid, cells, simplex, order, ncomp, jit, diri, neu, g = case
    m = _mesh(cells, simplex, jit)
    V = GT.lagrange_space(GT.interior(m), order, tensor_size=(ncomp,) if ncomp > 1 else None,
                          dirichlet_boundary=None if diri is None else GT.boundary(m, None if diri == "boundary" else diri))
    ref = _oracle_space(m, order, ncomp, diri)
    assert np.array_equal(V.face_dofs(), ref["cell_dofs"])
    b = GT.assemble_boundary_vector(g, GT.boundary(m, neu), V)
    ob = O.assemble_boundary_vector(ref, 2 * order, g, neu)
    assert b.shape == ob.shape
    if ob.size:
        assert np.abs(b - ob).max() <= 1e-12 * np.abs(ob).max()
