"""Request serving: assemble + solve requests with continuous batching.

A ``Server`` runs ``slots`` workers, each with its own context (its own CUDA
stream and buffer pool), so the device overlaps the work of concurrent
requests.  Requests arriving while others run are admitted as soon as a slot
is free and the HBM budget (sum of the admitted requests' estimated device
bytes) has room; a request whose estimate alone exceeds the budget is refused
with ``GT_ERR_BUDGET`` and counted.  Mesh, space and matrix stay on the
device for the life of a request.  Every kernel reduces in a fixed order per
request, so a request's result is bitwise the same alone and in any mix.

``request_stream`` draws the seeded request mix of the serving benchmark:
Poisson arrivals, each request Poisson or linear elasticity on Q1 or Q2
hexahedra, cell count log-uniform in a range, seeded per-cell coefficients.
"""
from __future__ import annotations

import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .api import (Context, assemble_matrix_and_vector, boundary, elasticity, interior, lagrange_space, laplacian,
                  solve, source)
from .mesh import cartesian_mesh, keyed_uniform, lognormal_cells


@dataclass
class Request:
    rid: int
    arrival: float      # seconds from the stream start
    form: str           # "poisson" | "elasticity"
    order: int
    cells_per_dir: int
    seed: int
    # filled by the server
    status: int = 0
    admitted: float = 0.0
    finished: float = 0.0
    iterations: int = 0
    rel_residual: float = 0.0
    solution: np.ndarray | None = field(default=None, repr=False)

    @property
    def cells(self):
        return self.cells_per_dir ** 3

    def est_bytes(self, precision="mixed"):
        m = self.order * self.cells_per_dir + 1
        nodes = m ** 3
        ncomp = 3 if self.form == "elasticity" else 1
        nnz = nodes * (2 * self.order + 1) ** 3 * ncomp * ncomp
        per = {"mixed": 16, "fp64": 12, "fp32": 8}[precision]
        return int(nnz * per + nodes * ncomp * 120 + self.cells * (24 + 8 + 4 * 27 * 3))


def request_stream(n, rate=2000.0, seed=505, min_cells=1e3, max_cells=2e6):
    """Seeded Poisson-process request stream."""
    u = keyed_uniform(seed, np.arange(4 * n, dtype=np.uint64))
    gaps = -np.log(1.0 - u[0::4]) / rate
    t = np.cumsum(gaps)
    form = np.where(u[1::4] < 0.5, "poisson", "elasticity")
    order = np.where(u[2::4] < 0.5, 1, 2)
    lo, hi = np.log(min_cells), np.log(max_cells)
    cells = np.exp(lo + (hi - lo) * u[3::4])
    k = np.maximum(2, np.round(cells ** (1.0 / 3.0))).astype(int)
    return [Request(i, float(t[i]), str(form[i]), int(order[i]), int(k[i]), seed * 1000003 + i) for i in range(n)]


def run_request(req: Request, ctx: Context, precision="mixed", rtol=1e-8, keep_solution=True):
    """Assemble and solve one request on ctx (mesh, space, matrix on the device)."""
    k = req.cells_per_dir
    m = cartesian_mesh((0, 1, 0, 1, 0, 1), (k, k, k))
    coef = lognormal_cells(m.num_cells, 0.5, req.seed)
    if req.form == "poisson":
        V = lagrange_space(interior(m), req.order, dirichlet_boundary=boundary(m), ctx=ctx)
        a, l = laplacian(coef), source(1.0)
    else:
        V = lagrange_space(interior(m), req.order, tensor_size=(3,), dirichlet_boundary=boundary(m, ["2-face-5"]),
                           ctx=ctx)
        a, l = elasticity(coef, 0.3), source([0.0, 0.0, -1.0])
    T = "mixed" if precision == "mixed" else np.float64
    A, b = assemble_matrix_and_vector(a, l, T, V)
    x, info = solve(A, b, rtol=rtol, mode="ir" if precision == "mixed" else "fp64", raise_on_fail=False)
    req.iterations = info["iterations"]
    req.rel_residual = info["rel_residual"]
    req.status = 0 if info["converged"] else _lib.GT_ERR_NOT_CONVERGED
    if keep_solution:
        req.solution = x
    del A, V
    return req


class Server:
    def __init__(self, slots=4, budget_bytes=150e9, precision="mixed", rtol=1e-8, device=0, keep_solutions=True,
                 ctx_factory=None, runner=None):
        self.slots = slots
        self.runner = runner or run_request
        self.budget = float(budget_bytes)
        self.precision = precision
        self.rtol = rtol
        self.keep = keep_solutions
        self.ctxs = [(ctx_factory or (lambda: Context(device)))() for _ in range(slots)]
        self.pending: list[Request] = []
        self.lock = threading.Condition()
        self.in_use = 0.0
        self.done: list[Request] = []
        self.refused: list[Request] = []
        self.closed = False
        self.t0 = None
        self.errors = []
        self.workers = [threading.Thread(target=self._work, args=(i,), daemon=True) for i in range(slots)]

    def _now(self):
        return time.perf_counter() - self.t0

    def submit(self, req: Request):
        with self.lock:
            if req.est_bytes(self.precision) > self.budget:
                req.status = _lib.GT_ERR_BUDGET
                req.admitted = req.finished = self._now()
                self.refused.append(req)
                return
            self.pending.append(req)
            self.lock.notify_all()

    def _take(self):
        with self.lock:
            while True:
                # first pending request that fits in the remaining budget
                for i, r in enumerate(self.pending):
                    need = r.est_bytes(self.precision)
                    if self.in_use + need <= self.budget:
                        self.pending.pop(i)
                        self.in_use += need
                        r.admitted = self._now()
                        return r, need
                if self.closed and not self.pending:
                    return None, 0
                self.lock.wait(0.05)

    def _work(self, slot):
        ctx = self.ctxs[slot]
        while True:
            req, need = self._take()
            if req is None:
                return
            try:
                self.runner(req, ctx, self.precision, self.rtol, self.keep)
            except Exception as e:  # a failed request is reported, the server continues
                req.status = getattr(e, "code", _lib.GT_ERR_CUDA)
                self.errors.append((req.rid, repr(e)))
            req.finished = self._now()
            # pooled blocks of a finished request are not counted against the
            # budget, so hand large pools back to the driver
            if ctx is not None and hasattr(ctx, "memory") and ctx.memory()[1] > self.budget / (4 * self.slots):
                ctx.trim()
            with self.lock:
                self.in_use -= need
                self.done.append(req)
                self.lock.notify_all()

    def serve(self, requests, realtime=True):
        """Feed requests at their arrival times; returns when all finished."""
        self.t0 = time.perf_counter()
        for w in self.workers:
            w.start()
        for r in sorted(requests, key=lambda r: r.arrival):
            if realtime:
                dt = r.arrival - self._now()
                if dt > 0:
                    time.sleep(dt)
            self.submit(r)
        with self.lock:
            self.closed = True
            self.lock.notify_all()
        for w in self.workers:
            w.join()
        return self.report()

    def report(self):
        done = [r for r in self.done if r.status == 0]
        lat = np.array([r.finished - r.arrival for r in done]) if done else np.array([0.0])
        span = max((r.finished for r in self.done), default=0.0)
        return {"completed": len(done), "failed": len(self.done) - len(done), "refused_budget": len(self.refused),
                "solves_per_s": len(done) / span if span > 0 else 0.0, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                "p99_ms": 1e3 * float(np.percentile(lat, 99)), "makespan_s": span,
                "errors": self.errors[:5]}
