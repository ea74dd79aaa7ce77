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
