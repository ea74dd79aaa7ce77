"""Batched assembly + solve of many independent problems.

``Batch`` wraps ``gt_batch_*``: the small instances (up to 32768 rows) are
solved by one persistent launch in which every CTA takes instances from a
queue (largest first) and runs each one's whole Jacobi-PCG alone; the large
instances, which fill the GPU by themselves, run one after the other through
the persistent cooperative solver.  Each instance keeps its own CG scalars
and a summation order that depends only on the instance.
``autotune_lanes`` picks the lanes per matrix row of the per-CTA SpMV by
timing the candidates on the batch itself and caches the choice in a JSON
file keyed by the batch's shape.

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
from .api import (Matrix, _ptr, assemble_matrix_and_vector, boundary, default_context, interior, lagrange_space,
                  laplacian, source)
from ._lib import check
from .mesh import cartesian_mesh, keyed_uniform, lognormal_cells

_MODES = {"fp64": _lib.GT_SOLVE_FP64, "ir": _lib.GT_SOLVE_IR, "mixed": _lib.GT_SOLVE_IR, "fp32": _lib.GT_SOLVE_FP32}


class Batch:
    def __init__(self, matrices, lanes: int | None = None):
        if not matrices:
            raise ValueError("empty batch")
        self.mats = list(matrices)
        self.ctx = self.mats[0].ctx
        arr = (C.c_void_p * len(self.mats))(*[m.h.value for m in self.mats])
        h = C.c_void_p()
        check(self.ctx.h, self.ctx.lib.gt_batch_create(self.ctx.h, len(self.mats), arr, C.byref(h)))
        self.h = h
        self.sizes = [m.shape[0] for m in self.mats]
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        if lanes:
            self.set_lanes(lanes)

    def set_lanes(self, lanes: int):
        check(self.ctx.h, self.ctx.lib.gt_batch_set_lanes(self.h, int(lanes)))

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
