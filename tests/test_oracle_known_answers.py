"""The CPU oracle against the known answers of the reference's own tests
(tests/golden/known_answers.json, each entry citing its file:line)."""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

import oracle as O

KA = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


def test_q2_unit_square_dof_counts():
    k = KA["q2_unit_square_boundary_dirichlet"]
    m = O.cartesian_mesh((0, 1, 0, 1), (1, 1))
    V = O.lagrange_space(m, k["order"], dirichlet="boundary")
    assert V["nfree"] == k["num_free_dofs"]
    assert V["ndiri"] == k["num_dirichlet_dofs"]


def test_sum_load_vector_and_mass():
    k1, k2 = KA["q1_2x2_sum_of_load_vector"], KA["q1_2x2_sum_of_mass_matrix"]
    m = O.cartesian_mesh((0, 1, 0, 1), (2, 2))
    V = O.lagrange_space(m, 1)
    b = O.assemble_vector(V, k1["degree"], 1.0)
    assert abs(b.sum() - k1["sum_b"]) < 1e-14
    _, _, nz = O.assemble_matrix(V, O.MASS, k2["degree"])
    assert abs(nz.sum() - k2["sum_A"]) < 1e-14


def test_integrals_on_0_2_square():
    k = KA["integral_x_plus_y_on_0_2_square"]
    m = O.cartesian_mesh((0, 2, 0, 2), (8, 8))
    V = O.lagrange_space(m, 1)
    b = O.assemble_vector(V, k["degree"], 1.0)
    assert abs(b.sum() - k["int_one"]) < 1e-13
    # x + y lies in Q1: int (x+y) = sum_i u_i int phi_i, u_i = x_i + y_i at the dof's node
    cd = V["cell_dofs"]
    u = np.zeros(V["nfree"])
    u[cd.reshape(-1) - 1] = m["coords"][m["cell_nodes"].reshape(-1) - 1].sum(1)
    assert abs(u @ b - k["int_x_plus_y"]) < 1e-13


def test_quadrature_weight_sums():
    k = KA["quadrature_weight_sums"]
    assert abs(O.quadrature(O.QUAD4, 2)[1].sum() - k["square_degree_2"]) < 1e-15
    assert abs(O.quadrature(O.HEX8, 4)[1].sum() - k["cube_degree_4"]) < 1e-15
    assert abs(O.quadrature(O.TET4, 2)[1].sum() - 1.0 / 6.0) < 1e-15


def test_reference_face_numbering():
    k = KA["q1_square_reference_faces"]
    assert O.QUAD_EDGES.tolist() == k["face_nodes_1"]


def _dof_values(m, V, fun):
    """Values of fun at the nodes of the free and Dirichlet dofs (Q_k on quads)."""
    order = V["order"]
    mm = order + 1
    cd = V["cell_dofs"]
    xf = np.zeros(V["nfree"])
    xd = np.zeros(V["ndiri"])
    for c in range(cd.shape[0]):
        X = m["coords"][m["cell_nodes"][c] - 1]
        for k in range(mm * mm):
            xi = np.array([k % mm, k // mm]) / order
            N = np.array([(1 - xi[0]) * (1 - xi[1]), xi[0] * (1 - xi[1]), (1 - xi[0]) * xi[1], xi[0] * xi[1]])
            val = fun(N @ X)
            d = cd[c, k]
            if d > 0:
                xf[d - 1] = val
            else:
                xd[-d - 1] = val
    return xf, xd


@pytest.mark.parametrize("case", KA["patch_tests_u_equals_x_plus_y"]["cases"], ids=lambda c: c["source"])
def test_patch_tests(case):
    tol = KA["patch_tests_u_equals_x_plus_y"]["tol"]
    m = O.cartesian_mesh(tuple(case["box"]), tuple(case["cells"]))
    V = O.lagrange_space(m, case["order"], dirichlet="boundary")
    deg = 2 * case["order"]
    cp, rv, nz = O.assemble_matrix(V, O.LAPLACE, deg)
    cpd, rvd, nzd = O.assemble_matrix(V, O.LAPLACE, deg, dirichlet_cols=True)
    A = sp.csc_matrix((nz, rv, cp), shape=(V["nfree"], V["nfree"]))
    Ad = sp.csc_matrix((nzd, rvd, cpd), shape=(V["nfree"], V["ndiri"]))
    uf, ud = _dof_values(m, V, lambda x: x.sum())
    b = O.assemble_vector(V, deg, 0.0) - Ad @ ud
    x = sla.spsolve(A, b)
    assert np.abs(x - uf).max() < tol


def test_oracle_pcg_matches_direct():
    m = O.cartesian_mesh((0, 1, 0, 1), (16, 16))
    V = O.lagrange_space(m, 1, dirichlet="boundary")
    cp, rv, nz = O.assemble_matrix(V, O.LAPLACE, 2)
    rp, ci, vv = O.csc_to_csr(cp, rv, nz, V["nfree"])
    b = O.assemble_vector(V, 2, 1.0)
    x, it, rr = O.pcg(rp, ci, vv, b, rtol=1e-13)
    xd = sla.spsolve(sp.csc_matrix((nz, rv, cp), shape=(V["nfree"],) * 2), b)
    assert rr < 1e-13 and np.abs(x - xd).max() / np.abs(xd).max() < 1e-11


# ---------------------------------------------------------------------------
# the oracle's Neumann term (assemble_in_Γn!, docs/src/src_jl/
# example_poisson_equation.jl:161-203): boundary measures, first moments and
# a Neumann patch test
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("cells,simplex,order,measure", [
    ((5, 4), False, 1, 8.0), ((3, 5), False, 2, 8.0), ((3, 2, 4), False, 1, 24.0), ((2, 3, 2), False, 2, 24.0),
    ((3, 2, 2), True, 1, 24.0), ((2, 2, 3), True, 2, 24.0)])
def test_neumann_term_sums_to_the_boundary_measure(cells, simplex, order, measure):
    # box [0,2]^D: perimeter 8, surface 24; interior nodes jittered
    m = O.cartesian_mesh(tuple(x for _ in cells for x in (0.0, 2.0)), cells, simplexify=simplex)
    O.jitter(m, 0.2, 5)
    V = O.lagrange_space(m, order)
    b = O.assemble_boundary_vector(V, 2 * order, 1.0)
    assert abs(b.sum() - measure) < 1e-12
    # one side only: x = 0 ("(D-1)-face-3" in 2-D, "(D-1)-face-5" in 3-D) has measure 2^(D-1)
    side = "1-face-3" if len(cells) == 2 else "2-face-5"
    bs = O.assemble_boundary_vector(V, 2 * order, 1.0, [side])
    assert abs(bs.sum() - 2.0 ** (len(cells) - 1)) < 1e-12


def test_neumann_term_first_moment():
    # Q1 reproduces u = x, so sum_i x_i b_i = int_dOmega x dGamma = 2 on the unit square
    m = O.cartesian_mesh((0, 1, 0, 1), (4, 3))
    V = O.lagrange_space(m, 1)
    b = O.assemble_boundary_vector(V, 2, 1.0)
    xf, _ = _dof_values(m, V, lambda x: x[0])
    assert abs(xf @ b - 2.0) < 1e-13


@pytest.mark.parametrize("order", [1, 2])
def test_neumann_patch_test(order):
    # -Laplace(u) = 0, u = x + y: Dirichlet on x = 0 (1-face-3), du/dn = 1 on
    # x = 1 (1-face-4) and y = 1 (1-face-2), du/dn = -1 on y = 0 (1-face-1)
    m = O.cartesian_mesh((0, 1, 0, 1), (4, 3))
    O.jitter(m, 0.15, 9)
    V = O.lagrange_space(m, order, dirichlet=["1-face-3"])
    deg = 2 * order
    cp, rv, nz = O.assemble_matrix(V, O.LAPLACE, deg)
    cpd, rvd, nzd = O.assemble_matrix(V, O.LAPLACE, deg, dirichlet_cols=True)
    A = sp.csc_matrix((nz, rv, cp), shape=(V["nfree"], V["nfree"]))
    Ad = sp.csc_matrix((nzd, rvd, cpd), shape=(V["nfree"], V["ndiri"]))
    uf, ud = _dof_values(m, V, lambda x: x.sum())
    b = (O.assemble_boundary_vector(V, deg, 1.0, ["1-face-4", "1-face-2"])
         + O.assemble_boundary_vector(V, deg, -1.0, ["1-face-1"]) - Ad @ ud)
    x = sla.spsolve(A, b)
    assert np.abs(x - uf).max() < 1e-10
