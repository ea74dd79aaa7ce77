"""Cell integrals on the GPU (gt_integrate, the restated GT.assemble_scalar)
against the reference's own known answers (integration and patch tests) and
against identities with the oracle-checked assembly: int u_h = u . b(f=1),
int u_h^2 = u' M u."""
import json
import os

import numpy as np
import pytest

import gtgpu as GT

pytestmark = pytest.mark.gpu

KA = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


def test_integral_known_answers():
    """test/integration_tests.jl:45-77: int (x+y) = 8 and int 1 = 4 on [0,2]^2"""
    ka = KA["integral_x_plus_y_on_0_2_square"]
    m = GT.cartesian_mesh((0.0, 2.0, 0.0, 2.0), (8, 8))
    V = GT.lagrange_space(GT.interior(m), 1)
    assert abs(GT.integrate(V, "volume") - ka["int_one"]) < 1e-12
    assert abs(GT.integrate(V, "poly", exact=GT.Polynomial(x=1.0, y=1.0)) - ka["int_x_plus_y"]) < 1e-12


def _unit_cube_int(p):
    c = p.c
    return c[0] + (c[1] + c[2] + c[3]) / 2 + (c[4] + c[5] + c[6]) / 3 + (c[7] + c[8] + c[9]) / 4


@pytest.mark.parametrize("case", ["p1tet_jitter", "p2tet_jitter", "q2hex", "q1hex"])
def test_quadratic_exact_on_affine_cells(case):
    """a quadratic is integrated exactly on affine cells (degree-2 rules)"""
    if case in ("p1tet_jitter", "p2tet_jitter"):
        m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (5, 4, 3), simplexify=True)
        GT.jitter_interior_nodes(m, 0.2, 3)
        V = GT.lagrange_space(GT.interior(m), 1 if case == "p1tet_jitter" else 2)
    else:
        m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (3, 4, 2))
        V = GT.lagrange_space(GT.interior(m), 2 if case == "q2hex" else 1)
    p = GT.Polynomial(c0=0.5, x=1.0, y=-2.0, z=0.25, xx=3.0, yy=-1.0, zz=2.0, xy=0.5, xz=-0.75, yz=1.5)
    assert abs(GT.integrate(V, "volume") - 1.0) < 1e-13
    assert abs(GT.integrate(V, "poly", exact=p) - _unit_cube_int(p)) < 1e-12


def test_field_integrals_match_assembled_vector_and_mass():
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (6, 5, 4), simplexify=True)
    GT.jitter_interior_nodes(m, 0.2, 5)
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    u = np.random.default_rng(8).standard_normal(V.num_free_dofs)
    b = GT.assemble_vector(GT.source(1.0), np.float64, V)
    M = GT.assemble_matrix(GT.mass(), np.float64, V, V).tocsr()
    ref1, ref2 = float(u @ b), float(u @ (M @ u))
    assert abs(GT.integrate(V, "field", u) - ref1) <= 1e-12 * max(1.0, abs(ref1))
    assert abs(GT.integrate(V, "l2_norm2", u) - ref2) <= 1e-12 * ref2


@pytest.mark.parametrize("case", KA["patch_tests_u_equals_x_plus_y"]["cases"], ids=lambda c: c["source"])
def test_patch_tests(case):
    """the reference's patch tests: u = x + y from its boundary values is
    reproduced (L2 and H1-seminorm errors, computed on the device)"""
    tol = KA["patch_tests_u_equals_x_plus_y"]["tol"]
    b0, b1, b2, b3 = case["box"]
    m = GT.cartesian_mesh((float(b0), float(b1), float(b2), float(b3)), tuple(case["cells"]))
    V = GT.lagrange_space(GT.interior(m), case["order"], dirichlet_boundary=GT.boundary(m))
    p = GT.Polynomial(x=1.0, y=1.0)
    xd = GT.interpolate_dirichlet(p, V)
    lp = GT.linear_problem(V, GT.laplacian(), GT.source(0.0), dirichlet_values=xd)
    if V.num_free_dofs:
        x, info = GT.solve(lp, rtol=1e-13, mode="fp64")
    else:
        x = np.zeros(0)
    assert GT.l2_error(V, x, p, xd) < tol
    assert GT.h1_error(V, x, p, xd) < tol


def test_patch_test_3d_tets_and_q2_quadratic():
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (4, 4, 3), simplexify=True)
    GT.jitter_interior_nodes(m, 0.2, 9)
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    p = GT.Polynomial(c0=1.0, x=1.0, y=2.0, z=3.0)
    xd = GT.interpolate_dirichlet(p, V)
    x, _ = GT.solve(GT.linear_problem(V, GT.laplacian(), GT.source(0.0), dirichlet_values=xd), rtol=1e-13)
    assert GT.l2_error(V, x, p, xd) < 1e-10 and GT.h1_error(V, x, p, xd) < 1e-9
    # Q2 reproduces u = x^2 + y with -lap u = -2
    m2 = GT.cartesian_mesh((0, 1, 0, 1), (5, 4))
    V2 = GT.lagrange_space(GT.interior(m2), 2, dirichlet_boundary=GT.boundary(m2))
    q = GT.Polynomial(y=1.0, xx=1.0)
    xd2 = GT.interpolate_dirichlet(q, V2)
    x2, _ = GT.solve(GT.linear_problem(V2, GT.laplacian(), GT.source(-2.0), dirichlet_values=xd2), rtol=1e-13)
    assert GT.l2_error(V2, x2, q, xd2) < 1e-10 and GT.h1_error(V2, x2, q, xd2) < 1e-9
    # P2 tets reproduce a quadratic: u = x^2 + yz + z, -lap u = -2
    m3 = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (3, 2, 2), simplexify=True)
    GT.jitter_interior_nodes(m3, 0.2, 13)
    V3 = GT.lagrange_space(GT.interior(m3), 2, dirichlet_boundary=GT.boundary(m3))
    s3 = GT.Polynomial(z=1.0, xx=1.0, yz=1.0)
    xd3 = GT.interpolate_dirichlet(s3, V3)
    x3, _ = GT.solve(GT.linear_problem(V3, GT.laplacian(), GT.source(-2.0), dirichlet_values=xd3), rtol=1e-13)
    assert GT.l2_error(V3, x3, s3, xd3) < 1e-10 and GT.h1_error(V3, x3, s3, xd3) < 1e-9
    # a P1 solution of the same quadratic problem is not exact: the error norm sees it
    V1 = GT.lagrange_space(GT.interior(m2), 1, dirichlet_boundary=GT.boundary(m2))
    xd1 = GT.interpolate_dirichlet(q, V1)
    x1, _ = GT.solve(GT.linear_problem(V1, GT.laplacian(), GT.source(-2.0), dirichlet_values=xd1), rtol=1e-13)
    assert GT.l2_error(V1, x1, q, xd1) > 1e-5


def test_integrate_rejects_bad_arguments():
    m = GT.cartesian_mesh((0, 1, 0, 1), (2, 2))
    V = GT.lagrange_space(GT.interior(m), 1)
    with pytest.raises(GT.GTError):
        GT.integrate(V, "l2_error2", np.zeros(V.num_free_dofs))  # no exact solution
    with pytest.raises(ValueError):
        GT.integrate(V, "field", np.zeros(3))


def test_solution_field():
    """GT.solution_field (src/problems.jl:501-526): the solved free values
    plus the Dirichlet field's values make the discrete field whose error
    norms the reference's tests check; solution_field(U, x) has zero
    Dirichlet values; solution_field! replaces the free values in place."""
    m = GT.cartesian_mesh((0, 1, 0, 1), (6, 5))
    GT.jitter_interior_nodes(m, 0.2, 3)
    V = GT.lagrange_space(GT.interior(m), 2, dirichlet_boundary=GT.boundary(m))
    p = GT.Polynomial(x=1.0, y=1.0)
    uhd = GT.dirichlet_field(V, p)
    assert np.array_equal(uhd.dirichlet_values, GT.interpolate_dirichlet(p, V))
    lp = GT.linear_problem(V, GT.laplacian(), GT.source(0.0), dirichlet_values=uhd)
    GT.solve(lp, rtol=1e-13)
    uh = GT.solution_field(uhd, lp)
    assert GT.l2_error(V, uh, p) < 1e-10 and GT.h1_error(V, uh, p) < 1e-10
    # the same field through the (free values, Dirichlet values) pair
    assert GT.l2_error(V, uh, p) == GT.l2_error(V, lp.x, p, uhd.dirichlet_values)
    # per-cell values: Dirichlet DOFs carry the interpolated data
    cd = V.face_dofs()
    dv = uh.dof_values()
    assert np.array_equal(dv[cd < 0], uhd.dirichlet_values[-cd[cd < 0] - 1])
    # zero Dirichlet values: the boundary data is missing, so the error is not small
    u0 = GT.solution_field(V, lp.x)
    assert not u0.dirichlet_values.any() and GT.l2_error(V, u0, p) > 1e-2
    # in place
    GT.solution_field_inplace(u0, np.zeros(V.num_free_dofs))
    assert GT.integrate(V, "l2_norm2", u0) == 0.0
    with pytest.raises(ValueError):
        GT.solution_field_inplace(u0, np.zeros(3))
