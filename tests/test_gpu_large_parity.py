"""Parity at the benchmark sizes, through the C ABI, against the oracle on
the same seeded inputs:

* the headline workload at full size -- 96^3 cubes x 6 jittered P1 tets
  (5,308,416 cells, 857,375 free DOFs), lognormal(0,1) kappa: DOF ids and CSR
  pattern bit-exact, FP64 values and load vector within 1e-12, the FP64 and
  mixed-precision solutions within 1e-8 of the oracle's FP64 solve;
* Q2 linear elasticity on HEX8 at 32^3 cells (the 64^3 benchmark size needs
  ~1.7e9 COO triplets, ~60 GB and minutes in the oracle; 32^3 is the largest
  it finishes in well under a minute): pattern bit-exact, FP64 values within
  1e-12, FP32 values within 2e-6, load vector within 1e-12;
* batched and served solutions: each instance's / request's solution within
  1e-8 of the oracle's FP64 solve of the same problem (oracle assembly, oracle
  CG to a 1e-13 relative residual), solved here to a 1e-10 relative
  residual, the tolerance the batched and served benchmarks use.
Errors are normwise: max |gpu - oracle| / max |oracle|."""
import numpy as np
import pytest

import gtgpu as GT
import oracle as O
from gtgpu import batch as GB
from gtgpu.server import Server, request_stream

pytestmark = pytest.mark.gpu

TOL64, TOL32, TOLX = 1e-12, 2e-6, 1e-8
RTOL = 1e-10


def _err(a, ref):
    return float(np.abs(np.asarray(a) - ref).max() / np.abs(ref).max())


def _oracle_space(m, order, ncomp, groups):
    om = dict(D=m.D, ctype=m.cell_type, coords=m.coords, cell_nodes=m.cell_nodes, pf0=m.corners,
              cells=m.cells_per_dir, box=m.domain)
    if m.D == 2:
        om["pf1"], om["pf1g"] = m.bfaces, m.bface_group
    else:
        om["pf1"], om["pf2"], om["pf2g"] = m.bedges, m.bfaces, m.bface_group
    return O.lagrange_space(om, order, ncomp=ncomp, dirichlet=groups)


def _oracle_solution(ref, form, order, coef, f, nu=0.3):
    cp, rv, nz = O.assemble_matrix(ref, form, 2 * order, coef=coef, nu=nu)
    orp, oci, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    ob = O.assemble_vector(ref, 2 * order, f)
    x, it, rr = O.pcg(orp, oci, ov, ob, rtol=1e-13, maxit=200000)
    assert rr <= 1e-13
    return x


def test_headline_workload_full_size():
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (96, 96, 96), simplexify=True)
    GT.jitter_interior_nodes(m, 0.2, 202)
    kappa = GT.lognormal_cells(m.num_cells, 1.0, 202)
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m))
    ref = _oracle_space(m, 1, 1, "boundary")
    assert V.num_free_dofs == ref["nfree"] == 857375
    assert np.array_equal(V.face_dofs(), ref["cell_dofs"])
    A, b = GT.assemble_matrix_and_vector(GT.laplacian(kappa), GT.source(1.0), "mixed", V)
    rp, ci, v = A.csr()
    cp, rv, nz = O.assemble_matrix(ref, O.LAPLACE, 2, coef=kappa)
    orp, oci, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert _err(v, ov) <= TOL64
    ob = O.assemble_vector(ref, 2, 1.0)
    assert _err(b, ob) <= TOL64
    xo, it, rr = O.pcg(orp, oci, ov, ob, rtol=1e-12)
    for mode in ("fp64", "ir"):
        x, info = GT.solve(A, b, rtol=RTOL, mode=mode)
        assert info["rel_residual"] <= RTOL
        assert _err(x, xo) <= TOLX, mode


def test_q2_elasticity_32():
    n = 32
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (n, n, n))
    V = GT.lagrange_space(GT.interior(m), 2, tensor_size=(3,), dirichlet_boundary=GT.boundary(m, ["2-face-5"]))
    ref = _oracle_space(m, 2, 3, ["2-face-5"])
    assert V.num_free_dofs == ref["nfree"]
    assert np.array_equal(V.face_dofs(), ref["cell_dofs"])
    a, f = GT.elasticity(1.0, 0.3), [0.0, 0.0, -1.0]
    A, b = GT.assemble_matrix_and_vector(a, GT.source(f), np.float64, V)
    rp, ci, v = A.csr()
    cp, rv, nz = O.assemble_matrix(ref, O.ELASTICITY, 4, coef=None, nu=0.3)
    orp, oci, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
    del cp, rv, nz
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    assert _err(v, ov) <= TOL64
    del rp, ci, v, A
    A32 = GT.assemble_matrix(a, np.float32, V)
    assert _err(A32.values32(), ov) <= TOL32
    ob = O.assemble_vector(ref, 4, f)
    assert _err(b, ob) <= TOL64


def test_batched_solutions_against_oracle():
    specs = [GB.InstanceSpec(0, 2, 1, 9), GB.InstanceSpec(1, 2, 2, 6), GB.InstanceSpec(2, 3, 1, 5),
             GB.InstanceSpec(3, 3, 2, 3), GB.InstanceSpec(4, 2, 1, 31), GB.InstanceSpec(5, 3, 1, 7),
             GB.InstanceSpec(6, 2, 2, 40), GB.InstanceSpec(7, 3, 2, 4), GB.InstanceSpec(8, 2, 1, 200)]
    inputs = [GB.instance_inputs(s, seed=404) for s in specs]
    inst = [GB.assemble_instance(s, seed=404, T="mixed", inputs=inp) for s, inp in zip(specs, inputs)]
    B = GB.Batch([A for _, _, A, _ in inst])
    assert B.info()["small_instances"] == len(specs) - 1  # the 201^2-row instance runs on the whole GPU
    x, infos = B.solve([b for _, _, _, b in inst], rtol=RTOL, mode="ir")
    for s, (m, kappa), xi, info in zip(specs, inputs, B.split(x), infos):
        assert info["rel_residual"] <= RTOL
        ref = _oracle_space(m, s.order, 1, "boundary")
        xo = _oracle_solution(ref, O.LAPLACE, s.order, kappa, 1.0)
        assert _err(xi, xo) <= TOLX, s


def test_served_solutions_against_oracle():
    reqs = request_stream(6, rate=2000.0, seed=17, min_cells=300, max_cells=3000)
    srv = Server(slots=3, budget_bytes=150e9, precision="mixed", rtol=RTOL)
    rep = srv.serve(reqs, realtime=True)
    srv.close()
    assert rep["completed"] == len(reqs)
    from gtgpu.mesh import cartesian_mesh, lognormal_cells
    for r in reqs:
        assert r.rel_residual <= RTOL
        k = r.cells_per_dir
        m = cartesian_mesh((0, 1, 0, 1, 0, 1), (k, k, k))
        coef = lognormal_cells(m.num_cells, 0.5, r.seed)
        if r.form == "poisson":
            ref = _oracle_space(m, r.order, 1, "boundary")
            xo = _oracle_solution(ref, O.LAPLACE, r.order, coef, 1.0)
        else:
            ref = _oracle_space(m, r.order, 3, ["2-face-5"])
            xo = _oracle_solution(ref, O.ELASTICITY, r.order, coef, [0.0, 0.0, -1.0])
        assert _err(r.solution, xo) <= TOLX, (r.form, r.order, k)
