"""Batched assembly + solve of many independent problems.

``Batch`` wraps ``gt_batch_*`` (scalar matrices, or block size 3 for 3-D
elasticity): the small instances (up to 32768 scalar rows) are
solved by one persistent launch in which every CTA takes instances from a
queue (largest first) and runs each one's whole Jacobi-PCG alone; the large
instances run through the single-system solver.  Each instance keeps its own
CG scalars and a summation order that depends only on the instance.
``run_batch`` drives a whole batch: HBM-budgeted waves, several worker
contexts assembling instances concurrently and solving the large ones on
their own streams while the small ones gather for the one-launch tier.
``autotune_lanes`` picks the lanes per matrix row of the per-CTA SpMV by
timing the candidates on the batch itself, ``autotune_batch`` the number of
worker contexts (and the lanes) on a sample of a workload; both cache the
choice in a JSON file keyed by the batch's shape.

``batch_workload`` draws the seeded instance list of the batched benchmark:
independent Poisson problems on unit boxes, dimension 2 or 3 and order 1 or 2
uniformly, cell counts log-uniform between two bounds, per-cell coefficient
lognormal(0, 0.5), homogeneous Dirichlet on the whole boundary.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import time
from dataclasses import dataclass

import numpy as np

from . import _lib
from .api import (Context, Matrix, _ptr, assemble_matrix_and_vector, boundary, default_context, interior,
                  lagrange_space, laplacian, solve, source)
from ._lib import check
from .mesh import cartesian_mesh, keyed_uniform, lognormal_cells

_MODES = {"fp64": _lib.GT_SOLVE_FP64, "ir": _lib.GT_SOLVE_IR, "mixed": _lib.GT_SOLVE_IR, "fp32": _lib.GT_SOLVE_FP32}


class Batch:
    """gt_batch over assembled matrices of one device, block size 1 or 3
    (they may come from several contexts); solved on ``ctx`` (default: the
    first matrix's)."""

    def __init__(self, matrices, lanes: int | None = None, ctx=None, small_rows: int | None = None):
        if not matrices:
            raise ValueError("empty batch")
        self.mats = list(matrices)
        self.ctx = ctx or self.mats[0].ctx
        arr = (C.c_void_p * len(self.mats))(*[m.h.value for m in self.mats])
        h = C.c_void_p()
        check(self.ctx.h, self.ctx.lib.gt_batch_create(self.ctx.h, len(self.mats), arr, C.byref(h)))
        self.h = h
        self.sizes = [m.shape[0] for m in self.mats]
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        if lanes:
            self.set_lanes(lanes)
        if small_rows is not None:
            self.set_small_rows(small_rows)

    def set_lanes(self, lanes: int):
        check(self.ctx.h, self.ctx.lib.gt_batch_set_lanes(self.h, int(lanes)))

    def set_small_rows(self, rows: int):
        """scalar rows up to which an instance is solved by one CTA (at most
        32768); larger instances of the batch's own context, up to 262,144
        rows, share grouped persistent launches (FP64 and mixed modes)"""
        check(self.ctx.h, self.ctx.lib.gt_batch_set_small_rows(self.h, int(rows)))

    def info(self):
        a = np.zeros(4, np.int64)
        check(self.ctx.h, self.ctx.lib.gt_batch_info(self.h, _ptr(a)))
        return dict(instances=int(a[0]), rows=int(a[1]), small_instances=int(a[2]), lanes=int(a[3]))

    def solve(self, b, rtol=1e-8, maxit=20000, mode="ir", raise_on_fail=True, out=None):
        """b: concatenated right-hand sides (numpy or device tensor) or a list of
        per-instance arrays.  Returns (x concatenated, list of info dicts)."""
        if isinstance(b, (list, tuple)):
            b = np.ascontiguousarray(np.concatenate([np.asarray(v, np.float64) for v in b]))
        x = out if out is not None else np.zeros(int(self.offsets[-1]), np.float64)
        infos = (_lib.SolveInfo * len(self.mats))()
        st = self.ctx.lib.gt_batch_solve(self.h, _ptr(b), _ptr(x), float(rtol), int(maxit), _MODES[mode], infos)
        if st != 0 and (raise_on_fail or st != _lib.GT_ERR_NOT_CONVERGED):
            check(self.ctx.h, st)
        return x, [dict(iterations=i.iterations, outer_iterations=i.outer_iterations, rel_residual=i.rel_residual,
                        fp64_iterations=i.fp64_iterations) for i in infos]

    def split(self, x):
        return [x[self.offsets[i]:self.offsets[i + 1]] for i in range(len(self.mats))]

    def signature(self) -> str:
        h = hashlib.sha1()
        for m in self.mats:
            h.update(np.array([m.shape[0], m.nnz], np.int64).tobytes())
        return h.hexdigest()[:16]

    def __del__(self):
        try:
            if self.h and self.ctx.h:
                self.ctx.lib.gt_batch_destroy(self.h)
        except Exception:
            pass


def _cache_path(path=None):
    return path or os.environ.get("GTGPU_AUTOTUNE_CACHE",
                                  os.path.join(os.path.expanduser("~"), ".cache", "gtgpu", "autotune.json"))


def autotune_lanes(batch: Batch, b, candidates=(1, 2, 4, 8), iters=48, cache=None, use_cache=True):
    """Pick the lanes per row of the batched SpMV by timing a short FP32 solve
    of the batch with each candidate; the result is cached by batch shape."""
    path = _cache_path(cache)
    key = batch.signature()
    table = {}
    if use_cache and os.path.exists(path):
        try:
            table = json.load(open(path))
        except Exception:
            table = {}
    if key in table:
        batch.set_lanes(table[key]["lanes"])
        return table[key]
    times = {}
    for g in candidates:
        batch.set_lanes(g)
        batch.solve(b, rtol=1e-30, maxit=16, mode="fp32", raise_on_fail=False)  # warm-up
        t0 = time.perf_counter()
        batch.solve(b, rtol=1e-30, maxit=iters, mode="fp32", raise_on_fail=False)
        times[g] = time.perf_counter() - t0
    best = min(times, key=times.get)
    batch.set_lanes(best)
    entry = {"lanes": best, "seconds": {str(k): v for k, v in times.items()}, "iters": iters}
    table[key] = entry
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        json.dump(table, open(path, "w"), indent=1)
    except OSError:
        pass
    return entry


@dataclass
class InstanceSpec:
    index: int
    dim: int
    order: int
    cells_per_dir: int


def batch_workload(n_instances=512, seed=404, min_cells=16 ** 2, max_cells=96 ** 3):
    """Seeded instance list: dim, order uniform; cells log-uniform in
    [min_cells, max_cells], per-direction n = max(2, round(cells^(1/dim)))."""
    u = keyed_uniform(seed, np.arange(4 * n_instances, dtype=np.uint64))
    dim = np.where(u[0::4] < 0.5, 2, 3)
    order = np.where(u[1::4] < 0.5, 1, 2)
    lo, hi = np.log(min_cells), np.log(max_cells)
    cells = np.exp(lo + (hi - lo) * u[2::4])
    n = np.maximum(2, np.round(cells ** (1.0 / dim))).astype(int)
    return [InstanceSpec(i, int(d), int(o), int(k)) for i, (d, o, k) in enumerate(zip(dim, order, n))]


def estimate_bytes(spec: InstanceSpec, precision="mixed"):
    """Device bytes of an assembled instance (matrix + vectors), an upper bound."""
    m = spec.order * spec.cells_per_dir + 1
    dofs = m ** spec.dim
    nnz = dofs * (2 * spec.order + 1) ** spec.dim
    per_nnz = {"mixed": 16, "fp64": 12, "fp32": 8}[precision]
    return int(nnz * per_nnz + dofs * 120 + (spec.cells_per_dir ** spec.dim) * 200)


def instance_inputs(spec: InstanceSpec, seed=404):
    """Host inputs of one batch instance: its mesh and its seeded cell
    coefficient."""
    box = tuple(x for _ in range(spec.dim) for x in (0.0, 1.0))
    m = cartesian_mesh(box, (spec.cells_per_dir,) * spec.dim)
    kappa = lognormal_cells(m.num_cells, 0.5, seed * 1000003 + spec.index)
    return m, kappa


def assemble_instance(spec: InstanceSpec, seed=404, T="mixed", ctx=None, inputs=None):
    """Mesh, space, matrix and load vector of one batch instance (from
    inputs = instance_inputs(spec, seed) when given; the mesh's device copy
    is made here, and dropped with mesh._device.clear() by a caller that
    keeps the host mesh)."""
    ctx = ctx or default_context()
    m, kappa = inputs if inputs is not None else instance_inputs(spec, seed)
    V = lagrange_space(interior(m), spec.order, dirichlet_boundary=boundary(m), ctx=ctx)
    A, b = assemble_matrix_and_vector(laplacian(kappa), source(1.0), T, V)
    return m, V, A, b


# ---------------------------------------------------------------------------
# concurrent batched assembly + solve
# ---------------------------------------------------------------------------
@dataclass
class BatchRun:
    """Outcome of run_batch: per-instance solutions (by instance index) and
    solve infos, plus the timings of the run."""
    solutions: dict
    infos: dict
    seconds: float
    waves: int
    small: int
    large: int


def waves_by_budget(specs, budget_bytes, precision="mixed"):
    """Instances largest first, greedily grouped so that each wave's estimated
    device bytes stay under the budget (an instance alone above it still
    forms a wave of its own)."""
    order = sorted(specs, key=lambda s: -estimate_bytes(s, precision))
    waves, cur, used = [], [], 0
    for s in order:
        e = estimate_bytes(s, precision)
        if cur and used + e > budget_bytes:
            waves.append(cur)
            cur, used = [], 0
        cur.append(s)
        used += e
    if cur:
        waves.append(cur)
    return waves


def run_batch(specs, inputs, precision="mixed", rtol=1e-10, maxit=100000, workers=4, small_rows=32768, lanes=None,
              budget_bytes=150e9, contexts=None, keep_solutions=True, ctx=None):
    """Batched assembly + solve of many independent instances.

    The instances go in HBM-budgeted waves (largest first).  In a wave,
    ``workers`` threads, each with its own context (its own CUDA streams and
    buffer pool), take instances from a largest-first queue and assemble them
    -- mesh upload, DOF numbering, sparsity, values (mixed: FP64-integrated
    FP64 values and FP32-integrated FP32 values) and load vector -- so the
    device overlaps the assembly of several instances.  An instance with more
    than ``small_rows`` rows is solved at once by its worker through the
    single-system solver on the worker's stream, so several such solves and
    the other workers' assembly run on the device together; the smaller
    instances wait for the wave's small tier: one gt_batch over all of them,
    solved by one persistent launch in which each CTA runs whole instances
    from a largest-first queue.  Every instance's arithmetic depends only on
    the instance, so its result is bitwise the same whatever the batch.

    inputs: {index: (mesh, kappa)} (instance_inputs).  precision "mixed"
    solves with FP32 CG + FP64 reliable updates (mode "ir"), float64 with
    FP64 CG.  Returns a BatchRun."""
    import threading

    T = "mixed" if precision == "mixed" else np.float64
    mode = "ir" if precision == "mixed" else "fp64"
    ctx = ctx or default_context()
    ctxs = list(contexts) if contexts else [Context(ctx.device) for _ in range(max(1, workers))]
    sols, infos = {}, {}
    n_small = n_large = 0
    t0 = time.perf_counter()
    waves = waves_by_budget(specs, budget_bytes, "mixed" if precision == "mixed" else "fp64")
    for wave in waves:
        queue = list(wave)  # largest first
        qlock = threading.Lock()
        small = []          # (spec, mesh, V, A, b) waiting for the small tier
        errors = []

        def work(wctx):
            while True:
                with qlock:
                    if not queue:
                        return
                    s = queue.pop(0)
                try:
                    m, kappa = inputs[s.index]
                    m_, V, A, b = assemble_instance(s, T=T, ctx=wctx, inputs=(m, kappa))
                    if A.shape[0] > small_rows:
                        x, info = solve(A, b, rtol=rtol, maxit=maxit, mode=mode, raise_on_fail=False)
                        with qlock:
                            sols[s.index] = x if keep_solutions else None
                            infos[s.index] = info
                        del A, V
                        m._device.pop(id(wctx), None)
                        if wctx.memory()[1] > budget_bytes / (4 * len(ctxs)):
                            wctx.trim()
                    else:
                        with qlock:
                            small.append((s, m, V, A, b))
                except Exception as e:  # reported after the wave
                    with qlock:
                        errors.append((s.index, e))

        threads = [threading.Thread(target=work, args=(c,)) for c in ctxs]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        if errors:
            raise errors[0][1]
        n_large += len(wave) - len(small)
        n_small += len(small)
        if small:
            small.sort(key=lambda t: t[0].index)
            B = Batch([A for _, _, _, A, _ in small], ctx=ctx)
            if lanes:
                B.set_lanes(lanes)
            x, binfo = B.solve([b for *_, b in small], rtol=rtol, maxit=maxit, mode=mode, raise_on_fail=False)
            for (s, m, V, A, b), xi, info in zip(small, B.split(x), binfo):
                sols[s.index] = xi.copy() if keep_solutions else None
                infos[s.index] = dict(info, converged=info["rel_residual"] <= rtol)
            del B
            for s, m, V, A, b in small:
                for c in ctxs:
                    m._device.pop(id(c), None)
            small.clear()
        for c in ctxs:
            c.trim()
    ctx.synchronize()
    seconds = time.perf_counter() - t0
    if not contexts:
        for c in ctxs:
            c.close()
    return BatchRun(sols, infos, seconds, len(waves), n_small, n_large)


def autotune_batch(specs, inputs, precision="mixed", rtol=1e-10, workers=(1, 2, 4, 8), sample=48, max_rows=2_000_000,
                   cache=None, use_cache=True, seed=0, small_rows=(4096, 16384, 32768)):
    """Pick run_batch's concurrency (worker contexts), the row limit of its
    one-CTA-per-instance tier (the tile of the batched kernel: an instance
    up to it is solved by one CTA, a larger one by the whole device) and
    the small tier's SpMV lanes for a workload: run_batch is timed on a
    seeded sample of the instances (at most ``sample``, each under
    ``max_rows`` rows, spread over the size range) once per worker count,
    then once per row limit with the best worker count, then autotune_lanes
    times the lane candidates on the sample's small tier.  The choice is
    cached in the autotune JSON file under the workload's signature."""
    path = _cache_path(cache)
    sig = hashlib.sha1(repr(sorted((s.dim, s.order, s.cells_per_dir) for s in specs)).encode()).hexdigest()[:16]
    key = f"batch2:{precision}:{sig}"
    table = {}
    if use_cache and os.path.exists(path):
        try:
            table = json.load(open(path))
        except Exception:
            table = {}
    if key in table:
        return table[key]
    rows = {s.index: (s.order * s.cells_per_dir - 1) ** s.dim for s in specs}
    pool = sorted([s for s in specs if rows[s.index] <= max_rows], key=lambda s: rows[s.index])
    if len(pool) > sample:
        pick = np.linspace(0, len(pool) - 1, sample).round().astype(int)
        pool = [pool[i] for i in sorted(set(pick.tolist()))]
    sub = {s.index: inputs[s.index] for s in pool}
    run_batch(pool[:4], sub, precision, rtol=rtol, workers=1)  # warm-up (module load, pools)
    times = {}
    for w in workers:
        times[w] = run_batch(pool, sub, precision, rtol=rtol, workers=w, keep_solutions=False).seconds
    best_w = min(times, key=times.get)
    tiers = {}
    for sr in small_rows:
        tiers[sr] = run_batch(pool, sub, precision, rtol=rtol, workers=best_w, small_rows=sr,
                              keep_solutions=False).seconds
    best_sr = min(tiers, key=tiers.get)
    ctx = default_context()
    T = "mixed" if precision == "mixed" else np.float64
    small = [s for s in pool if rows[s.index] <= best_sr]
    lanes = 0
    if small:
        inst = [assemble_instance(s, T=T, ctx=ctx, inputs=sub[s.index]) for s in small]
        B = Batch([A for _, _, A, _ in inst])
        lanes = autotune_lanes(B, np.concatenate([b for *_, b in inst]), iters=32, cache=cache, use_cache=use_cache)["lanes"]
        del B, inst
    entry = {"workers": int(best_w), "small_rows": int(best_sr), "lanes": int(lanes),
             "seconds": {str(k): v for k, v in times.items()},
             "small_rows_seconds": {str(k): v for k, v in tiers.items()}, "sample": len(pool)}
    table = {}
    if os.path.exists(path):
        try:
            table = json.load(open(path))
        except Exception:
            table = {}
    table[key] = entry
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        json.dump(table, open(path, "w"), indent=1)
    except OSError:
        pass
    return entry
