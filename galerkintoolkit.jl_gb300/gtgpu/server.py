"""Request serving: assemble + solve requests with continuous batching.

A ``Server`` runs ``slots`` workers, each with its own context (its own CUDA
streams and buffer pool), so the device overlaps the work of concurrent
requests.  Requests arriving while others run wait in a pending set and are
admitted as soon as a slot is free and the HBM budget has room for their
estimated device bytes; a request whose estimate alone exceeds the budget is
refused with ``GT_ERR_BUDGET`` and counted.  The policy picks the next
pending request: ``"sjf"`` the smallest estimated work (the default: under a
stream the device cannot keep up with it completes the most requests),
``"fifo"`` the earliest arrival.  The next request waits until the budget
has room for it.

State stays on the device across requests: every slot keeps a cache of
resident geometries keyed by (form, order, mesh) -- the mesh's device copy,
the space (DOF numbering) and the assembled matrix (sparsity and value
arrays) -- up to its share of the budget, least recently used out first.  A
request for a cached geometry only refills the values and the load vector
(GT.update_matrix_and_vector!, src/problems.jl:409-414) before its solve; a
miss builds mesh, space and pattern and caches them.  Host meshes come from
a ``MeshLibrary`` of pre-built meshes, so no mesh is generated inside a
request's latency.  Every kernel reduces in a fixed order per request, and a
refill gives bitwise the values of a fresh assembly, so a request's result
is bitwise the same alone, in any mix, hit or miss.

Continuous batching: a slot that takes a request of at most ``batch_rows``
scalar rows (Poisson or elasticity; by default 2,048) also takes the other
such requests pending at that moment (up to ``batch_max``, within the
budget) and solves them together with ``gt_batch``: those up to
``small_rows`` rows one CTA each in one persistent launch per block size,
larger ones (when ``batch_rows`` admits them) in shared grouped persistent
launches, each on the CTAs its own solve would use.  So a stream of small
requests is not served one grid-wide solve at a time, and a request's result
never depends on its batch: the one-CTA tier's depends on the request alone,
the grouped tier's is bitwise that of the request's own solve.

``request_stream`` draws the seeded request mix of the serving benchmark:
Poisson arrivals, each request Poisson or linear elasticity on Q1 or Q2
hexahedra, cell count log-uniform in a range, seeded per-cell coefficients
(lognormal(0, 0.5), generated on the slot's device stream from the seed:
gt_lognormal_cells).
"""
from __future__ import annotations

import heapq
import threading
import time
from collections import OrderedDict, deque
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .api import (Context, assemble_matrix_and_vector, boundary, elasticity, interior, lagrange_space, laplacian,
                  lognormal_cells_device, solve, source, update_matrix_and_vector)
from .mesh import cartesian_mesh, keyed_uniform


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
    cache_hit: bool = False
    solution: np.ndarray | None = field(default=None, repr=False)

    @property
    def cells(self):
        return self.cells_per_dir ** 3

    @property
    def key(self):
        return (self.form, self.order, self.cells_per_dir)

    @property
    def ncomp(self):
        return 3 if self.form == "elasticity" else 1

    def est_bytes(self, precision="mixed"):
        m = self.order * self.cells_per_dir + 1
        nodes = m ** 3
        ncomp = self.ncomp
        nnz = nodes * (2 * self.order + 1) ** 3 * ncomp * ncomp
        per = {"mixed": 16, "fp64": 12, "fp32": 8}[precision]
        return int(nnz * per + nodes * ncomp * 120 + self.cells * (24 + 8 + 4 * 27 * 3))

    @property
    def rows(self):
        """free block rows (the homogeneous Dirichlet boundary removed)"""
        m = self.order * self.cells_per_dir - 1
        return m ** 3 if self.form == "poisson" else (self.order * self.cells_per_dir) * m * m

    @property
    def scalar_rows(self):
        return self.rows * self.ncomp

    def est_work(self):
        """Relative cost of the solve: matrix entries x a CG iteration count
        growing with the nodes per direction (x4 for elasticity's ratio of
        iterations)."""
        m = self.order * self.cells_per_dir + 1
        nnz = m ** 3 * (2 * self.order + 1) ** 3 * self.ncomp ** 2
        return nnz * m * (4.0 if self.form == "elasticity" else 1.0)


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


class MeshLibrary:
    """Pre-built host meshes of the unit cube, one per cells-per-direction
    (built once, shared read-only by every slot)."""

    def __init__(self, ks=()):
        self.meshes = {}
        self.lock = threading.Lock()
        for k in sorted(set(ks)):
            self.get(k)

    def get(self, k):
        with self.lock:
            m = self.meshes.get(k)
            if m is None:
                m = cartesian_mesh((0, 1, 0, 1, 0, 1), (k, k, k))
                self.meshes[k] = m
        return m


@dataclass
class _Entry:
    V: object
    A: object
    bytes: int


class GeometryCache:
    """One slot's resident geometries: key -> the instances (space, matrix)
    kept for it -- several when requests of one geometry run in one batch,
    each taking its own -- least recently used keys out first when the
    cached bytes pass the capacity."""

    def __init__(self, ctx, capacity_bytes):
        self.ctx = ctx
        self.capacity = float(capacity_bytes)
        self.entries: OrderedDict = OrderedDict()
        self.bytes = 0
        self.hits = 0
        self.misses = 0

    def acquire(self, key, taken):
        """a cached instance of key not in taken (ids), or None"""
        lst = self.entries.get(key)
        if lst:
            for e in lst:
                if id(e) not in taken:
                    self.entries.move_to_end(key)
                    self.hits += 1
                    taken.add(id(e))
                    return e
        return None

    def put(self, key, V, A, nbytes, library, taken):
        self.misses += 1
        if nbytes > self.capacity:
            return False
        while self.entries and self.bytes + nbytes > self.capacity:
            self._evict(library)
        e = _Entry(V, A, nbytes)
        self.entries.setdefault(key, []).append(e)
        taken.add(id(e))
        self.bytes += nbytes
        return True

    def uses_mesh(self, k):
        return any(key[2] == k for key in self.entries)

    def _evict(self, library):
        key, lst = self.entries.popitem(last=False)
        self.bytes -= sum(e.bytes for e in lst)
        del lst
        if not self.uses_mesh(key[2]):  # the mesh's device copy goes with its last entry
            library.get(key[2])._device.pop(id(self.ctx), None)

    def clear(self, library):
        while self.entries:
            self._evict(library)


def _forms(req, coef):
    if req.form == "poisson":
        return laplacian(coef), source(1.0)
    return elasticity(coef, 0.3), source([0.0, 0.0, -1.0])


def _assemble(req: Request, ctx, precision, cache, library, taken=None):
    """The request's matrix and load vector on ctx: refilled in the slot's
    cache when its geometry is resident, else mesh upload, space and
    assembly (then cached when it fits the slot's share).  Returns (A, b,
    release) with release() dropping what nothing resident keeps."""
    m = library.get(req.cells_per_dir)
    coef = lognormal_cells_device(m.num_cells, 0.5, req.seed, ctx)  # generated on the slot's stream
    a, l = _forms(req, coef)
    T = "mixed" if precision == "mixed" else np.float64
    taken = set() if taken is None else taken
    e = cache.acquire(req.key, taken) if cache is not None else None
    if e is not None:
        A, b = update_matrix_and_vector(e.A, a, l)
        req.cache_hit = True
    else:
        if req.form == "poisson":
            V = lagrange_space(interior(m), req.order, dirichlet_boundary=boundary(m), ctx=ctx)
        else:
            V = lagrange_space(interior(m), req.order, tensor_size=(3,), dirichlet_boundary=boundary(m, ["2-face-5"]),
                               ctx=ctx)
        A, b = assemble_matrix_and_vector(a, l, T, V)
        if cache is None or not cache.put(req.key, V, A, req.est_bytes(precision), library, taken):
            del V

    def release():
        if cache is None or (e is None and not cache.uses_mesh(req.cells_per_dir)):
            m._device.pop(id(ctx), None)  # nothing resident keeps this mesh's device copy
    return A, b, release


def _record(req, x, info, rtol, keep_solution):
    req.iterations = info["iterations"]
    req.rel_residual = info["rel_residual"]
    req.status = 0 if info["rel_residual"] <= rtol else _lib.GT_ERR_NOT_CONVERGED
    if keep_solution:
        req.solution = x


def run_request(req: Request, ctx: Context, precision="mixed", rtol=1e-8, keep_solution=True, cache=None,
                library=None):
    """Assemble (or refill) and solve one request on ctx."""
    A, b, release = _assemble(req, ctx, precision, cache, library or MeshLibrary())
    x, info = solve(A, b, rtol=rtol, maxit=200000, mode="ir" if precision == "mixed" else "fp64",
                    raise_on_fail=False)
    _record(req, x, info, rtol, keep_solution)
    del A
    release()
    return req


def run_batch_requests(reqs, ctx: Context, precision="mixed", rtol=1e-8, keep_solution=True, cache=None,
                       library=None, small_rows=2048):
    """Assemble (or refill) several requests on ctx and solve them together
    (gt_batch): those up to small_rows scalar rows one CTA each in one
    persistent launch per block size, the larger ones in grouped persistent
    launches (each on the CTAs its own solve would use)."""
    from .batch import Batch
    library = library or MeshLibrary()
    taken = set()  # cached instances handed to this batch: one per request
    built = [_assemble(r, ctx, precision, cache, library, taken) for r in reqs]
    B = Batch([A for A, _, _ in built], ctx=ctx, small_rows=small_rows)
    x, infos = B.solve([b for _, b, _ in built], rtol=rtol, maxit=200000,
                       mode="ir" if precision == "mixed" else "fp64", raise_on_fail=False)
    for r, xi, info in zip(reqs, B.split(x), infos):
        _record(r, xi.copy() if keep_solution else None, info, rtol, keep_solution)
    del B
    for A, b, release in built:
        del A
        release()
    return reqs


class Server:
    def __init__(self, slots=4, budget_bytes=150e9, precision="mixed", rtol=1e-8, device=0, keep_solutions=True,
                 ctx_factory=None, runner=None, policy="sjf", cache_fraction=0.1, library=None, batching=True,
                 batch_max=16, batch_rows=2048, small_rows=2048):
        self.slots = slots
        self.runner = runner or run_request
        self.budget = float(budget_bytes)
        self.precision = precision
        self.rtol = rtol
        self.keep = keep_solutions
        self.policy = policy
        # requests up to batch_rows scalar rows go through gt_batch (alone
        # or with others, up to batch_max); batching=False: one grid-wide
        # solve per request.  In a batch, requests up to small_rows are
        # solved by one CTA each, so that tier lasts as long as its largest
        # member: the limit keeps it short (on GB300, under the 2000 req/s
        # stream, 2048 scalar rows and batches of 16 completed 1.8x the
        # requests of 32768 and 64 at a p50 of 10 ms instead of 0.4 s); the
        # larger ones, when batch_rows lets them in, share grouped persistent
        # launches, each bitwise its own solve.  Measured with batch_rows
        # 262,144: 588 requests/s at a p50 of 138 ms against 604 at 9.3 ms
        # (a batch then waits for its grouped launches, and requests of one
        # geometry in one batch each need their own resident instance), so
        # by default only the one-CTA requests are batched
        self.batching = batching and runner is None
        self.batch_max = max(1, batch_max)
        self.batch_rows = batch_rows
        self.small_rows = small_rows
        self.library = library or MeshLibrary()
        self.ctxs = [(ctx_factory or (lambda: Context(device)))() for _ in range(slots)]
        # each slot caches geometries up to its share of cache_fraction of the
        # budget; that share is reserved, so admission counts it as in use
        cached = runner is None
        share = self.budget * cache_fraction / max(1, slots)
        self.caches = [GeometryCache(c, share) if cached else None for c in self.ctxs]
        self.reserved = share * slots if cached else 0.0
        # pending requests: a heap by estimated work (sjf) or arrival order (fifo)
        self.pending = [] if policy == "sjf" else deque()
        self.lock = threading.Condition()
        self.in_use = 0.0
        self.done: list[Request] = []
        self.refused: list[Request] = []
        self.closed = False
        self.deadline = None
        self.t0 = None
        self.errors = []
        self.workers = [threading.Thread(target=self._work, args=(i,), daemon=True) for i in range(slots)]

    def _now(self):
        return time.perf_counter() - self.t0

    def submit(self, req: Request):
        with self.lock:
            if req.est_bytes(self.precision) > self.budget - self.reserved:
                req.status = _lib.GT_ERR_BUDGET
                req.admitted = req.finished = self._now()
                self.refused.append(req)
                return
            if self.policy == "sjf":
                heapq.heappush(self.pending, (req.est_work(), req.arrival, req.rid, req))
            else:
                self.pending.append(req)
            self.lock.notify_all()

    def _batchable(self, r):
        return self.batching and r.scalar_rows <= self.batch_rows

    def _pop_next(self):
        """the next request by the policy if the budget has room for it"""
        if not self.pending:
            return None
        r = self.pending[0][3] if self.policy == "sjf" else self.pending[0]
        if self.in_use + self.reserved + r.est_bytes(self.precision) > self.budget:
            return None
        if self.policy == "sjf":
            heapq.heappop(self.pending)
        else:
            self.pending.popleft()
        self.in_use += r.est_bytes(self.precision)
        r.admitted = self._now()
        return r

    def _take(self):
        """a list of requests to run together (one, or a batch of small
        ones) and their budget bytes"""
        with self.lock:
            while True:
                if self.deadline is not None and self._now() >= self.deadline:
                    return None, 0
                r = self._pop_next()
                if r is not None:
                    got = [r]
                    if self._batchable(r):
                        # the small requests at the head of the queue join it
                        while len(got) < self.batch_max and self.pending:
                            nxt = self.pending[0][3] if self.policy == "sjf" else self.pending[0]
                            if not self._batchable(nxt):
                                break
                            q = self._pop_next()
                            if q is None:
                                break
                            got.append(q)
                    return got, sum(q.est_bytes(self.precision) for q in got)
                if self.closed and not self.pending:
                    return None, 0
                self.lock.wait(0.01)

    def _work(self, slot):
        ctx = self.ctxs[slot]
        cache = self.caches[slot]
        while True:
            reqs, need = self._take()
            if reqs is None:
                return
            try:
                if self._batchable(reqs[0]):  # a batch of one too: the result never depends on the batch
                    run_batch_requests(reqs, ctx, self.precision, self.rtol, self.keep, cache=cache,
                                       library=self.library, small_rows=self.small_rows)
                elif cache is not None:
                    self.runner(reqs[0], ctx, self.precision, self.rtol, self.keep, cache=cache, library=self.library)
                else:
                    self.runner(reqs[0], ctx, self.precision, self.rtol, self.keep)
            except Exception as e:  # a failed request is reported, the server continues
                for req in reqs:
                    req.status = getattr(e, "code", _lib.GT_ERR_CUDA)
                self.errors.append((reqs[0].rid, repr(e)))
            now = self._now()
            for req in reqs:
                req.finished = now
            # pooled blocks of a finished request are not counted against the
            # budget, so hand large pools back to the driver
            if ctx is not None and hasattr(ctx, "memory") and ctx.memory()[1] > self.budget / (4 * self.slots):
                ctx.trim()
            with self.lock:
                self.in_use -= need
                self.done.extend(reqs)
                self.lock.notify_all()

    def serve(self, requests, realtime=True, duration=None):
        """Feed requests at their arrival times (realtime) and serve them.
        duration (seconds from the start): requests arriving later are not
        fed and no request starts after it; those still waiting then are
        reported as pending.  Returns the report."""
        self.t0 = time.perf_counter()
        self.deadline = duration
        for w in self.workers:
            w.start()
        for r in sorted(requests, key=lambda r: r.arrival):
            if duration is not None and r.arrival >= duration:
                break
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

    def close(self):
        """Drops the cached geometries and the slots' contexts."""
        for c in self.caches:
            if c is not None:
                c.clear(self.library)
        for c in self.ctxs:
            if hasattr(c, "close"):
                c.close()

    def report(self):
        done = [r for r in self.done if r.status == 0]
        lat = np.array([r.finished - r.arrival for r in done]) if done else np.array([0.0])
        span = max((r.finished for r in self.done), default=0.0)
        return {"completed": len(done), "failed": len(self.done) - len(done), "refused_budget": len(self.refused),
                "pending_at_end": len(self.pending), "solves_per_s": len(done) / span if span > 0 else 0.0,
                "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
                "makespan_s": span, "cache_hits": sum(1 for r in done if r.cache_hit), "policy": self.policy,
                "slots": self.slots, "errors": self.errors[:5]}
