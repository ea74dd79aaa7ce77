"""Host logic of the request server (admission by HBM budget, refusal,
continuous batching, latency accounting) with a fake runner: no GPU."""
import threading
import time

import numpy as np

from gtgpu import _lib
from gtgpu.server import Request, Server, request_stream


def test_request_stream_is_seeded_and_in_range():
    a = request_stream(50, rate=2000.0, seed=505)
    b = request_stream(50, rate=2000.0, seed=505)
    assert [(r.form, r.order, r.cells_per_dir, r.arrival) for r in a] == \
           [(r.form, r.order, r.cells_per_dir, r.arrival) for r in b]
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0) and 0.0 < arr[-1] < 0.2
    assert all(9 <= r.cells_per_dir <= 127 for r in a)
    assert {r.form for r in a} == {"poisson", "elasticity"} and {r.order for r in a} == {1, 2}


def test_admission_respects_budget_and_refuses_oversize():
    live = []
    peak = [0.0]
    lock = threading.Lock()

    def runner(req, ctx, precision, rtol, keep):
        with lock:
            live.append(req.est_bytes(precision))
            peak[0] = max(peak[0], sum(live))
        time.sleep(0.01)
        with lock:
            live.remove(req.est_bytes(precision))
        req.status = 0

    reqs = [Request(i, 0.001 * i, "poisson", 1, 20, i) for i in range(12)]
    big = Request(99, 0.0, "elasticity", 2, 120, 1)
    budget = 3.5 * reqs[0].est_bytes("mixed")
    srv = Server(slots=4, budget_bytes=budget, ctx_factory=lambda: None, runner=runner)
    rep = srv.serve(reqs + [big], realtime=True)
    assert rep["completed"] == 12 and rep["refused_budget"] == 1
    assert big.status == _lib.GT_ERR_BUDGET
    assert peak[0] <= budget  # never more than three requests of this size at once
    assert rep["p99_ms"] >= rep["p50_ms"] > 0


def test_failed_request_does_not_stop_the_server():
    def runner(req, ctx, precision, rtol, keep):
        if req.rid == 2:
            raise RuntimeError("simulated device failure")
        req.status = 0

    reqs = [Request(i, 0.0, "poisson", 1, 10, i) for i in range(5)]
    srv = Server(slots=2, budget_bytes=1e12, ctx_factory=lambda: None, runner=runner)
    rep = srv.serve(reqs, realtime=False)
    assert rep["completed"] == 4 and rep["failed"] == 1
    assert rep["errors"][0][0] == 2
