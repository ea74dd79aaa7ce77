"""Non-homogeneous Dirichlet data (GT.PartitionedSolvers_linear_problem with
uhd, src/problems.jl:439-453): the lifted load vector b - Ad xd against the
oracle's free x Dirichlet matrix Ad, and linear fields reproduced exactly by
the solve (the reference's patch tests, test/assembly_tests.jl:43-118,
test/problems_tests.jl:85-100, with Dirichlet data u = x + y)."""
import numpy as np
import pytest
import scipy.sparse as sp

import gtgpu as GT
import oracle as O
from test_gpu_parity import _build, _KIND

pytestmark = pytest.mark.gpu

LIFT_CASES = [
    # (id, cells, simplex, order, ncomp, dirichlet groups, form, jitter, coef sigma)
    ("p1tet_jitter", (5, 4, 4), True, 1, 1, "boundary", O.LAPLACE, 0.2, 1.0),
    ("q1hex_jitter_x0", (5, 4, 3), False, 1, 1, ["2-face-5"], O.LAPLACE, 0.15, 1.0),
    ("q2quad_jitter", (5, 4), False, 2, 1, "boundary", O.LAPLACE, 0.2, 0.5),
    ("q2hex_elast_affine", (3, 3, 4), False, 2, 3, ["2-face-5"], O.ELASTICITY, 0.0, 0.5),
    ("q1quad_elast_affine", (5, 4), False, 1, 2, ["1-face-3"], O.ELASTICITY, 0.0, 0.5),
    ("q1hex_elast_jitter", (4, 3, 3), False, 1, 3, ["2-face-5"], O.ELASTICITY, 0.1, 0.5),
    ("q2hex_lap_affine", (3, 3, 3), False, 2, 1, "boundary", O.LAPLACE, 0.0, 1.0),
]


def _field(X, ncomp):
    """A smooth nonlinear Dirichlet field (scalar or vector)."""
    base = np.sin(1.3 * X[:, 0]) + X[:, 1] ** 2 - (0.7 * X[:, 2] if X.shape[1] > 2 else 0.0)
    if ncomp == 1:
        return base
    return np.stack([base * (k + 1) + 0.1 * k for k in range(ncomp)], axis=1)


@pytest.mark.parametrize("case", LIFT_CASES, ids=[c[0] for c in LIFT_CASES])
def test_lifted_vector_matches_oracle(case):
    m, V, ref, a, coef, form, order = _build(case)
    ncomp = V.ncomp
    xd = GT.interpolate_dirichlet(lambda X: _field(X, ncomp), V)
    f = [0.3 * (k + 1) for k in range(ncomp)] if ncomp > 1 else 1.0
    p = GT.linear_problem(V, a, GT.source(f), np.float64, dirichlet_values=xd)
    b0 = O.assemble_vector(ref, 2 * order, f)
    cp, rv, nz = O.assemble_matrix(ref, form, 2 * order, coef=coef, nu=0.3, dirichlet_cols=True)
    Ad = sp.csc_matrix((nz, rv, cp), shape=(ref["nfree"], ref["ndiri"]))
    want = b0 - Ad @ xd
    scale = max(np.abs(b0).max(), np.abs(Ad @ xd).max())
    assert np.abs(p.b - want).max() <= 1e-12 * scale
    # the matrix of the lifted problem is the plain one
    A = GT.assemble_matrix(a, np.float64, V, V)
    assert np.array_equal(A.csr()[2], p.A.csr()[2])


PATCH_CASES = [
    ("p1tet_jitter", (4, 4, 3), True, 1, 1, "boundary", O.LAPLACE, 0.2, 0.0),
    ("q1hex", (4, 3, 3), False, 1, 1, "boundary", O.LAPLACE, 0.0, 0.0),
    ("q2hex_affine", (3, 3, 2), False, 2, 1, "boundary", O.LAPLACE, 0.0, 0.0),
    ("q2quad", (4, 5), False, 2, 1, "boundary", O.LAPLACE, 0.0, 0.0),
    ("q2hex_elast_affine", (2, 3, 2), False, 2, 3, "boundary", O.ELASTICITY, 0.0, 0.0),
]


@pytest.mark.parametrize("case", PATCH_CASES, ids=[c[0] for c in PATCH_CASES])
def test_linear_field_reproduced(case):
    """u linear (Laplace, kappa = 1, f = 0; elasticity with constant strain
    and no body force) is an exact discrete solution on affine cells: the
    solve with the interpolated Dirichlet data returns u at the free nodes."""
    m, V, ref, a, coef, form, order = _build(case)
    D, ncomp = m.D, V.ncomp
    W = np.array([[0.7, -1.1, 0.4], [0.2, 0.5, -0.3], [-0.6, 0.1, 0.9]])[:ncomp, :D]

    def u(X):
        v = X @ W.T + 0.25
        return v[:, 0] if ncomp == 1 else v

    xd = GT.interpolate_dirichlet(u, V)
    f = [0.0] * ncomp if ncomp > 1 else 0.0
    p = GT.linear_problem(V, a, GT.source(f), np.float64, dirichlet_values=xd)
    x, info = GT.solve(p, rtol=1e-13, maxit=20000, mode="fp64")
    free, _ = V.node_coordinates()
    want = np.asarray(u(free), np.float64).reshape(-1)
    assert np.abs(x - want).max() <= 1e-9 * max(1.0, np.abs(want).max())
