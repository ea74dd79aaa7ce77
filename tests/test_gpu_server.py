"""Serving on the GPU: each request's solution is bitwise the same served
alone (one slot, one request at a time) and in a concurrent mix."""
import numpy as np
import pytest

from gtgpu.server import Server, request_stream

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_the_mix():
    reqs_a = request_stream(8, rate=2000.0, seed=11, min_cells=500, max_cells=8000)
    reqs_b = request_stream(8, rate=2000.0, seed=11, min_cells=500, max_cells=8000)
    s1, s4 = Server(slots=1, budget_bytes=150e9), Server(slots=4, budget_bytes=150e9)
    alone = s1.serve(reqs_a, realtime=False)
    mixed = s4.serve(reqs_b, realtime=True)
    s1.close()
    s4.close()
    assert alone["completed"] == 8 and mixed["completed"] == 8
    for ra, rb in zip(sorted(reqs_a, key=lambda r: r.rid), sorted(reqs_b, key=lambda r: r.rid)):
        assert ra.rel_residual <= 1e-8
        assert np.array_equal(ra.solution, rb.solution)


def test_cached_geometry_refill_is_bitwise_a_fresh_assembly():
    """A slot keeps a served request's geometry (mesh, space, pattern) on the
    device; a later request on the same geometry only refills the values and
    the load vector, and its solution is bitwise that of a slot that builds
    everything afresh."""
    from gtgpu.server import Request
    reqs = [Request(0, 0.0, "poisson", 2, 7, 101), Request(1, 0.0, "elasticity", 1, 6, 102),
            Request(2, 0.0, "poisson", 2, 7, 103), Request(3, 0.0, "elasticity", 1, 6, 104)]
    # batches of two: requests 2 and 3 come after the batch that cached their geometries
    warm = Server(slots=1, budget_bytes=150e9, rtol=1e-10, policy="fifo", batch_max=2)
    warm.serve(reqs, realtime=False)
    assert [r.cache_hit for r in sorted(reqs, key=lambda r: r.rid)] == [False, False, True, True]
    fresh = [Request(r.rid, 0.0, r.form, r.order, r.cells_per_dir, r.seed) for r in reqs[2:]]
    cold = Server(slots=1, budget_bytes=150e9, rtol=1e-10, policy="fifo", cache_fraction=1e-9, batch_max=2)
    cold.serve(fresh, realtime=False)
    for a, b in zip(sorted(reqs[2:], key=lambda r: r.rid), sorted(fresh, key=lambda r: r.rid)):
        assert not b.cache_hit and a.rel_residual <= 1e-10
        assert np.array_equal(a.solution, b.solution)
    warm.close()
    cold.close()


def test_serving_window_reports_pending():
    """duration: no request starts after the window; those left are pending"""
    reqs = request_stream(200, rate=2000.0, seed=5, min_cells=20000, max_cells=60000)
    srv = Server(slots=2, budget_bytes=150e9, rtol=1e-8, keep_solutions=False)
    rep = srv.serve(reqs, realtime=True, duration=0.05)
    srv.close()
    fed = sum(1 for r in reqs if r.arrival < 0.05)
    assert rep["completed"] + rep["pending_at_end"] + rep["failed"] + rep["refused_budget"] == fed
    assert rep["pending_at_end"] > 0


def test_batched_small_requests_with_shared_geometry():
    """Small Poisson and elasticity requests pending together are solved in
    one persistent launch per block size; requests on the same geometry in
    one batch each take their own resident instance.  Every result is
    bitwise that of the request served alone, and within 1e-10 in residual."""
    from gtgpu.server import Request
    def reqs():
        return [Request(i, 0.0, "elasticity" if i % 4 == 3 else "poisson", 1 + (i % 2),
                        4 if i % 4 == 3 else (9 if i % 2 == 0 else 5), 300 + i) for i in range(8)]
    together, alone = reqs(), reqs()
    s1 = Server(slots=1, budget_bytes=150e9, rtol=1e-10, policy="fifo")
    rep = s1.serve(together, realtime=False)
    s2 = Server(slots=1, budget_bytes=150e9, rtol=1e-10, policy="fifo", batch_max=1)
    s2.serve(alone, realtime=False)
    assert rep["completed"] == 8
    for a, b in zip(together, alone):
        assert a.rel_residual <= 1e-10
        assert np.array_equal(a.solution, b.solution)
    s1.close()
    s2.close()


def test_device_coefficients_match_host_generator():
    """gt_lognormal_cells: the served requests' coefficients generated on the
    device equal the host generator's up to the last bits of log/cos/exp."""
    import gtgpu as GT
    for n, seed in ((1, 7), (1000, 505000003), (123457, 2 ** 40 + 3)):
        d = GT.lognormal_cells_device(n, 0.5, seed).numpy()
        h = GT.lognormal_cells(n, 0.5, seed)
        assert np.all(d > 0) and np.abs(d - h).max() <= 1e-14 * np.abs(h).max()


def test_batched_medium_requests_are_bitwise_their_own_solves():
    """Requests above the one-CTA limit are batched into grouped persistent
    launches; each result is bitwise that of the same request served with
    batching off (one persistent solve per request).  Those up to the limit
    (one CTA each) agree within the tolerance."""
    from gtgpu.server import Request
    def reqs():
        return [Request(i, 0.0, "elasticity" if i % 3 == 2 else "poisson", 1 + (i % 2), (14, 10, 8, 12, 16, 7)[i],
                        700 + i) for i in range(6)]
    a, b = reqs(), reqs()
    s1 = Server(slots=1, budget_bytes=150e9, rtol=1e-10, policy="fifo", batch_rows=262144)
    rep = s1.serve(a, realtime=False)
    s2 = Server(slots=1, budget_bytes=150e9, rtol=1e-10, policy="fifo", batching=False)
    s2.serve(b, realtime=False)
    s1.close()
    s2.close()
    assert rep["completed"] == 6
    assert any(r.scalar_rows > 2048 for r in a)
    for ra, rb in zip(a, b):
        assert ra.rel_residual <= 1e-10
        if ra.scalar_rows > 2048:
            assert np.array_equal(ra.solution, rb.solution), (ra.form, ra.order, ra.cells_per_dir)
        else:
            assert np.abs(ra.solution - rb.solution).max() <= 1e-8 * np.abs(rb.solution).max()
