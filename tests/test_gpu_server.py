"""Serving on the GPU: each request's solution is bitwise the same served
alone (one slot, one request at a time) and in a concurrent mix."""
import numpy as np
import pytest

from gtgpu.server import Server, request_stream

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_the_mix():
    reqs_a = request_stream(8, rate=2000.0, seed=11, min_cells=500, max_cells=8000)
    reqs_b = request_stream(8, rate=2000.0, seed=11, min_cells=500, max_cells=8000)
    alone = Server(slots=1, budget_bytes=150e9).serve(reqs_a, realtime=False)
    mixed = Server(slots=4, budget_bytes=150e9).serve(reqs_b, realtime=True)
    assert alone["completed"] == 8 and mixed["completed"] == 8
    for ra, rb in zip(sorted(reqs_a, key=lambda r: r.rid), sorted(reqs_b, key=lambda r: r.rid)):
        assert ra.rel_residual <= 1e-8
        assert np.array_equal(ra.solution, rb.solution)
