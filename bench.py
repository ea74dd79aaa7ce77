#!/usr/bin/env python
"""Benchmark of the finite-element assembly + solve path on GB300.

Workload (default): 3-D Poisson on jittered tetrahedra -- unit cube, 96^3
cubes split into 6 tets (5,308,416 cells, 857,375 free DOFs), interior nodes
jittered U(-0.2h, 0.2h) (seed 202), P1, 4-point Strang quadrature, per-cell
coefficient lognormal(0,1) (seed 202), homogeneous Dirichlet on the whole
boundary, plain FP64.  One step = GT.assemble_matrix + GT.assemble_vector from
the device-resident space: sparsity (incidence + pattern), FP64 integration,
deterministic scatter and the load vector.  Metric: nnz assembled per second.

`e2e` measures the same step through the C ABI with host buffers: the node
coordinates and the coefficient are copied in from pinned host memory and
the CSR arrays and the vector are read back into pinned host memory, every
step.  The JSON line also carries the roofline of the dominant kernel, the
CPU baseline (the oracle restatement of the reference algorithm on the
host's cores), the solve rates (plain FP64 PCG vs FP32 PCG with FP64 reliable
updates), the HBM rooflines of the scatter and of the FP64 SpMV, and the SM
clocks sampled during the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

N > 1 runs N independent replicas (the path is assembled per mesh; there is
no data-path exchange), launched by torch.distributed.run.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "galerkintoolkit.jl_gb300"))

METRIC = "nnz/s assembled (assemble_matrix + assemble_vector, plain FP64)"
SOLVE_RTOL = 1e-10   # relative residual of the headline solves (FP64 and mixed)
SOLVE_SAMPLES = 100  # timed solves per mode (p50 / p99 latency)
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}
# DRAM bytes (read + write) per launch on the default workload (96^3 x 6 P1
# tets), from one-pass ncu captures of the full workload (summaries under
# profiles/): the double-float element kernel, the scatter and the FP64 SpMV
# (sliced-ELL copy)
TRAFFIC: dict = {"elements": 149.65e6 + 532.88e6,
                 "scatter": 826.09e6 + 97.81e6,
                 "spmv": 159.938048e6 + 5.819904e6}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    p.add_argument("--cells", type=int, default=96, help="cubes per direction (96 = the benchmark workload)")
    p.add_argument("--no-solve", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--workload", default="tets", choices=["tets", "elasticity", "batched", "serving"],
                   help="tets: the headline workload; the others measure the remaining configurations")
    p.add_argument("--instances", type=int, default=512, help="batched: number of instances")
    p.add_argument("--serve-seconds", type=float, default=30.0, help="serving: length of the request stream")
    p.add_argument("--slots", type=int, default=4, help="serving: concurrent request slots")
    p.add_argument("--budget-gb", type=float, default=150.0, help="batched/serving: HBM admission budget")
    return p.parse_args()


# ---------------------------------------------------------------------------
# other configurations (one JSON line each; not the driver's headline)
# ---------------------------------------------------------------------------
def cpu_elasticity(n):
    """The oracle's FP64 assembly (counting pass, COO append, COO -> CSC, and
    the load vector) of the elasticity problem on a bounded n^3 sample, on
    all host cores and on one (the reference is single-threaded), in nnz/s:
    the per-nonzero rate carries over to the full size (its COO, ~60 GB at
    64^3, does not fit the host)."""
    O = _oracle()
    from gtgpu.mesh import cartesian_mesh
    m = cartesian_mesh((0, 1, 0, 1, 0, 1), (n, n, n))
    om = dict(D=3, ctype=m.cell_type, coords=m.coords, cell_nodes=m.cell_nodes, pf0=m.corners, pf1=m.bedges,
              pf2=m.bfaces, pf2g=m.bface_group, cells=m.cells_per_dir, box=m.domain)
    ref = O.lagrange_space(om, 2, ncomp=3, dirichlet=["2-face-5"])
    out = {"unit": "nnz/s", "kind": "port", "sample": f"{n}^3 HEX8 Q2 elasticity, FP64, one repetition"}
    for key, th in (("value", os.cpu_count()), ("single_thread", 1)):
        O.set_threads(th)
        t0 = time.perf_counter()
        _, rv, _ = O.assemble_matrix(ref, O.ELASTICITY, 4, coef=None, nu=0.3)
        O.assemble_vector(ref, 4, [0.0, 0.0, -1.0])
        dt = time.perf_counter() - t0
        if key == "value":
            out.update({"value": rv.size / dt, "cores": O.num_threads(), "nnz": int(rv.size), "seconds": dt})
        else:
            out["single_thread"] = {"value": rv.size / dt, "cores": 1, "seconds": dt}
    return out


def run_elasticity(args):
    """3-D linear elasticity, 64^3 HEX8 cells, Q2 vector space (6.39M free
    DOFs), E=1, nu=0.3, body force (0,0,-1), clamped at x=0, 3x3x3 Gauss.
    Assembly in FP64, FP32 and mixed; solves: plain FP64 PCG and FP64
    refinement around FP32 PCG to 1e-10; the CPU baseline (the oracle) on a
    12^3 sample, per nonzero."""
    import torch
    import gtgpu as GT
    n = args.cells if args.cells != 96 else 64
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (n, n, n))
    ctx = GT.Context(0)
    V = GT.lagrange_space(GT.interior(m), 2, tensor_size=(3,), dirichlet_boundary=GT.boundary(m, ["2-face-5"]),
                          ctx=ctx)
    a, l = GT.elasticity(1.0, 0.3), GT.source([0.0, 0.0, -1.0])
    out = {"metric": "Q2 elasticity: nnz/s assembled and solve time, mixed vs plain FP64", "n_gpus": 1,
           "config": {"workload": f"3-D linear elasticity, {n}^3 HEX8, Q2 vector (3 comp), E=1 nu=0.3, clamped x=0",
                      "free_dofs": V.num_free_dofs}, "data": "synthetic (seeded)"}
    res = {}
    for T in (np.float64, np.float32, "mixed"):
        name = {np.float64: "fp64", np.float32: "fp32", "mixed": "mixed"}[T]
        ts = []
        for _ in range(max(2, args.warmup)):
            ctx.synchronize()
            t0 = time.perf_counter()
            A, b = GT.assemble_matrix_and_vector(a, l, T, V)
            ctx.synchronize()
            ts.append(time.perf_counter() - t0)
            if name != "mixed":
                del A
        res[name] = {"assemble_ms": 1e3 * min(ts), "nnz": A.nnz if name == "mixed" else None}
    nnz = A.nnz
    for k in res:
        res[k]["nnz_per_s"] = nnz / (res[k]["assemble_ms"] * 1e-3)
    A32 = GT.assemble_matrix(a, np.float32, V, V)
    v32 = A32.values32().astype(np.float64)
    _, _, v64 = A.csr()
    res["fp32_values_rel_err_vs_fp64"] = float(np.abs(v32 - v64).max() / np.abs(v64).max())
    del A32, v32
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_elasticity(12)
    if args.no_solve:
        out.update({"assembly": res, "nnz": int(nnz)})
        print(json.dumps(out), flush=True)
        return
    sol = {}
    xs = {}
    for mode in ("fp64", "ir"):
        t0 = time.perf_counter()
        x, info = GT.solve(A, b, rtol=1e-10, maxit=200000, mode=mode, raise_on_fail=False)
        sol[mode] = {"solve_s": time.perf_counter() - t0, **info}
        xs[mode] = x
    sol["ir_vs_fp64_rel_err"] = float(np.abs(xs["ir"] - xs["fp64"]).max() / np.abs(xs["fp64"]).max())
    out.update({"assembly": res, "solve": sol, "nnz": int(nnz)})
    print(json.dumps(out), flush=True)


def run_batched(args):
    """512 independent Poisson instances (dim 2|3, order 1|2, cells
    log-uniform 16^2..96^3, kappa lognormal(0,0.5), Dirichlet boundary),
    each assembled and solved to a 1e-8 relative residual (the
    configuration's tolerance; the largest instances' eps64 * cond(A) puts
    1e-10 out of FP64's reach).  Three arms time
    the upload, DOF numbering, assembly and solve of every instance (the host
    meshes and seeded coefficients are generated before the timed region):
      mixed_batched  gtgpu.batch.run_batch, mixed precision (FP32-integrated
                     FP32 values + FP64 values; FP32 CG with FP64 reliable
                     updates): worker contexts assembling concurrently, large
                     instances solved on the workers' streams, the small ones
                     in one persistent launch
      fp64_batched   the same runner in plain FP64
      plain_fp64     one instance at a time on one context, FP64 assembly and
                     FP64 CG
    The worker count, the one-CTA tier's row limit and the small tier's SpMV
    lanes come from autotune_batch (untimed, cached).  Solutions of a seeded sample of the
    instances are compared with the oracle's FP64 solve."""
    import gtgpu as GT
    from gtgpu import batch as GB
    rtol = 1e-8  # the configuration's tolerance (FP64 cannot reach 1e-10 on its largest instances)
    specs = GB.batch_workload(args.instances, seed=404)
    budget = args.budget_gb * 1e9
    ctx = GT.default_context()
    host = {s.index: GB.instance_inputs(s, seed=404) for s in specs}  # untimed: the inputs
    tune = GB.autotune_batch(specs, host, "mixed", rtol=rtol)
    ctx.trim()
    runs = {}
    for name, prec in (("mixed_batched", "mixed"), ("fp64_batched", "fp64")):
        r = GB.run_batch(specs, host, prec, rtol=rtol, workers=tune["workers"], lanes=tune["lanes"],
                         small_rows=tune["small_rows"], budget_bytes=budget)
        its = [i["iterations"] for i in r.infos.values()]
        runs[name] = {"solves_per_s": len(specs) / r.seconds, "seconds": r.seconds, "waves": r.waves,
                      "small_tier": r.small, "large_tier": r.large,
                      "worst_rel_residual": max(i["rel_residual"] for i in r.infos.values()),
                      "iterations_sum": int(sum(its)),
                      "fp64_iterations_sum": int(sum(i.get("fp64_iterations", 0) for i in r.infos.values())),
                      "instances_handed_to_fp64": int(sum(1 for i in r.infos.values()
                                                          if prec == "mixed" and i.get("fp64_iterations", 0) > 0))}
        runs[name]["_sol"] = r.solutions
        ctx.trim()
    # plain FP64 path, one instance at a time
    t0 = time.perf_counter()
    worst64, its64, plain_sol = 0.0, [], {}
    for s in specs:
        m, V, A, b = GB.assemble_instance(s, seed=404, T=np.float64, ctx=ctx, inputs=host[s.index])
        x, info = GT.solve(A, b, rtol=rtol, maxit=100000, mode="fp64", raise_on_fail=False)
        its64.append(info["iterations"])
        worst64 = max(worst64, info["rel_residual"])
        plain_sol[s.index] = x
        del A, V
        host[s.index][0]._device.clear()
        if ctx.memory()[1] > 20e9:
            ctx.trim()
    t_plain = time.perf_counter() - t0
    runs["plain_fp64"] = {"solves_per_s": len(specs) / t_plain, "seconds": t_plain, "worst_rel_residual": worst64,
                          "iterations_sum": int(sum(its64)), "_sol": plain_sol}
    # oracle check on a seeded sample (instances the oracle solves in seconds)
    O = _oracle()
    rows = {s.index: (s.order * s.cells_per_dir - 1) ** s.dim for s in specs}
    cand = [s for s in specs if rows[s.index] <= 40000]
    pick = np.linspace(0, len(cand) - 1, min(24, len(cand))).round().astype(int)
    errs = {k: 0.0 for k in runs}
    for i in sorted(set(pick.tolist())):
        s = cand[i]
        m, kappa = host[s.index]
        om = dict(D=m.D, ctype=m.cell_type, coords=m.coords, cell_nodes=m.cell_nodes, pf0=m.corners)
        if m.D == 2:
            om["pf1"], om["pf1g"] = m.bfaces, m.bface_group
        else:
            om["pf1"], om["pf2"], om["pf2g"] = m.bedges, m.bfaces, m.bface_group
        ref = O.lagrange_space(om, s.order, dirichlet="boundary")
        cp, rv, nz = O.assemble_matrix(ref, O.LAPLACE, 2 * s.order, coef=kappa)
        orp, oci, ov = O.csc_to_csr(cp, rv, nz, ref["nfree"])
        xo, _, _ = O.pcg(orp, oci, ov, O.assemble_vector(ref, 2 * s.order, 1.0), rtol=1e-13, maxit=200000)
        for k in runs:
            errs[k] = max(errs[k], _relerr(runs[k]["_sol"][s.index], xo))
    for k in runs:
        del runs[k]["_sol"]
    out = {"metric": "batched solves/s (assemble + solve to 1e-8), mixed batched vs plain FP64", "n_gpus": 1,
           "config": {"workload": f"{args.instances} Poisson instances, dim 2|3, Q1|Q2, cells log-uniform 16^2..96^3",
                      "budget_gb": args.budget_gb, "rtol": rtol, "tuning": tune},
           **runs,
           "speedup_vs_plain_fp64": runs["plain_fp64"]["seconds"] / runs["mixed_batched"]["seconds"],
           "speedup_vs_fp64_batched": runs["fp64_batched"]["seconds"] / runs["mixed_batched"]["seconds"],
           "oracle_check": {"instances": int(len(set(pick.tolist()))), "max_rel_err": errs,
                            "reference": "oracle assembly + oracle FP64 PCG to 1e-13",
                            "error_scale": "max |gpu - oracle| / max |oracle|"},
           "data": "synthetic (seeded)"}
    print(json.dumps(out), flush=True)


def run_serving(args):
    """Open-loop Poisson-process stream (mean 2000 req/s) of assemble+solve
    requests: Poisson or elasticity, Q1|Q2 hexahedra, cells log-uniform
    1e3..2e6, seeded coefficients, HBM admission budget 150 GB, solved to a
    1e-10 relative residual.  The stream runs for --serve-seconds: requests
    arriving in that window are fed at their arrival times, none starts after
    it, and those still waiting then are reported as pending (the offered
    load is far above what one GPU completes, so the window, not a request
    count, bounds the run).  Arms: the served path in mixed precision and
    in FP64 (--slots slots, geometries kept resident and values refilled on
    a repeat, requests of up to 2048 scalar rows solved in batches of up to
    16 in one persistent launch, coefficients generated on the device), and
    the plain FP64 path (one slot, no resident state, one solve per
    request).  Host meshes come from a library built before the stream.
    p50/p99 latency = arrival -> result, over the completed requests."""
    from gtgpu.server import MeshLibrary, Server, request_stream
    rate, dur = 2000.0, args.serve_seconds
    n = int(rate * dur * 1.2) + 16
    reqs0 = [r for r in request_stream(n, rate=rate, seed=505) if r.arrival < dur]
    lib = MeshLibrary(r.cells_per_dir for r in reqs0)  # untimed: the pre-built meshes
    res = {}
    arms = (("mixed", args.slots, "mixed", {}), ("fp64", args.slots, "fp64", {}),
            ("plain_fp64", 1, "fp64", {"cache_fraction": 1e-12, "batching": False}))
    for name, slots, prec, kw in arms:
        reqs = request_stream(n, rate=rate, seed=505)
        srv = Server(slots=slots, budget_bytes=args.budget_gb * 1e9, precision=prec, rtol=1e-10,
                     keep_solutions=False, library=lib, **kw)
        res[name] = srv.serve(reqs, realtime=True, duration=dur)
        srv.close()
    out = {"metric": "serving: solves/s and p50/p99 latency, mixed served path vs plain FP64 (and FP64 with the same features)",
           "n_gpus": 1,
           "config": {"workload": f"Poisson arrivals 2000/s for {dur:g} s ({len(reqs0)} requests), cells log-uniform "
                                  f"1e3..2e6, Poisson|elasticity x Q1|Q2", "budget_gb": args.budget_gb,
                      "rtol": 1e-10, "policy": "shortest estimated work first", "slots": args.slots},
           **res,
           "speedup_vs_plain_fp64": res["mixed"]["solves_per_s"] / max(res["plain_fp64"]["solves_per_s"], 1e-12),
           "speedup_vs_fp64_same_features": res["mixed"]["solves_per_s"] / max(res["fp64"]["solves_per_s"], 1e-12),
           "data": "synthetic (seeded)"}
    print(json.dumps(out), flush=True)


class L2Flush:
    """Flushes L2 (129 MB on GB300) between timed launches: a 256 MiB write,
    then a 256 MiB read of a second buffer, so the dirty lines of the write
    are written back before the timed work starts and it meets a cold, clean
    L2 (as a kernel that follows unrelated work does, and as ncu measures)."""

    def __init__(self):
        import torch
        self.w = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        self.r = torch.ones(64 << 20, dtype=torch.float32, device="cuda")

    def __call__(self):
        self.w.fill_(1)
        self.sink = self.r.sum()


def spmv_roofline(A, flush, stream, traffic=None, reps=20):
    """y = A x with the FP64 SpMV (gt_spmv, device vectors; on the sliced-ELL
    copy the library keeps for scalar matrices, built by the first call), L2
    flushed before each launch, timed by the library's phase marks (CUDA
    events on its stream right before and after the kernel); algorithmic
    bytes = those of the CSR matrix: values + column indices + row pointers
    + x + y (the copy's padding and slice pointers are not counted)."""
    import torch
    from gtgpu.api import _ptr
    n = A.shape[0]
    x = torch.ones(n, dtype=torch.float64, device="cuda")
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    ctx = A.ctx
    ts = []
    for i in range(reps + 3):
        flush()
        ctx.profile_begin()
        ctx.lib.gt_spmv(A.h, _ptr(x), _ptr(y))
        ph = dict(ctx.profile_end())
        if i >= 3:
            ts.append(ph["spmv"])
    ms = statistics.median(ts)
    nb = A.nnz * (8 + 4) + (n + 1) * 8 + 2 * n * 8
    return {"kernel": "k_spmv_sell<double, double>", "achieved": nb / (ms * 1e-3) / 1e9, "unit": "GB/s",
            "algorithmic_bytes": nb, "ms": ms, "traffic": traffic}


def workload(n):
    import gtgpu as GT
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (n, n, n), simplexify=True)
    GT.jitter_interior_nodes(m, 0.2, 202)
    kappa = GT.lognormal_cells(m.num_cells, 1.0, 202)
    return m, kappa


def wl_config(n, extra=None):
    c = {"workload": f"3-D Poisson, unit cube {n}^3 cubes x 6 P1 tets ({6 * n ** 3} cells), jittered +-0.2h, "
                     f"kappa lognormal(0,1), Dirichlet on the boundary, plain FP64",
         "cells": 6 * n ** 3, "order": 1, "quadrature": "Strang 4-point", "seed": 202,
         "l2": "flushed between timed steps (256 MiB write, then 256 MiB read of another buffer)",
         "element_arithmetic": "FP64 values; P1 element matrices in double-float (FP32 pairs) unless GTGPU_P1=fp64"}
    if extra:
        c.update(extra)
    return c


class Replicas:
    """The N > 1 layout of the benchmark: N independent replicas of the
    step, one process per GPU (the path assembles one mesh per process and
    has no data-path exchange).  The only collectives are the barriers around
    the timed region and the max over ranks of the step time; the throughput
    is the units all ranks processed divided by that time (weak scaling)."""

    def __init__(self, backend="nccl"):
        import torch.distributed as dist
        self.dist = dist
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        if self.world > 1 and not dist.is_initialized():
            dist.init_process_group(backend)

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max_ms(self, ms, device):
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        if self.world > 1:
            self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def value(self, units_per_rank, ms):
        return self.world * units_per_rank / (ms * 1e-3)

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return dict(PEAKS_FALLBACK), "fallback"


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join("/tmp", f"gt_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 8 and f[0].replace(".", "").isdigit():
                    rows.append(f)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[0]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][1]), "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------------------
# CPU side: the oracle restatement of the reference algorithm
# ---------------------------------------------------------------------------
def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    return O


def oracle_space(m):
    """The oracle's space of the benchmark mesh (DOF numbering; not timed:
    the GPU step also starts from the space)."""
    O = _oracle()
    om = dict(D=3, ctype=O.TET4, coords=m.coords, cell_nodes=m.cell_nodes, pf0=m.corners, pf1=m.bedges,
              pf2=m.bfaces, pf2g=m.bface_group)
    return O.lagrange_space(om, 1, dirichlet="boundary")


def cpu_assembly(m, kappa, reps=1, threads=None, space=None):
    """Times the oracle's assemble_matrix (counting pass + COO append +
    COO->CSC) + assemble_vector on the host's cores (threads: OpenMP
    threads, 1 = the reference's single-threaded path).  Returns nnz, the
    times, the threads used and the last (colptr, rowval, nzval, b)."""
    O = _oracle()
    O.set_threads(threads or os.cpu_count())
    V = space if space is not None else oracle_space(m)
    times, out = [], None
    for _ in range(reps):
        t = time.perf_counter()
        cp, rv, nz = O.assemble_matrix(V, O.LAPLACE, 2, coef=kappa)
        b = O.assemble_vector(V, 2, 1.0)
        times.append(time.perf_counter() - t)
        out = (cp, rv, nz, b)
    return out[1].size, times, O.num_threads(), out


def _relerr(a, ref):
    ref = np.asarray(ref)
    scale = float(np.abs(ref).max()) if ref.size else 0.0
    return float(np.abs(np.asarray(a) - ref).max() / scale) if scale > 0 else 0.0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.cells
    m, kappa = workload(n)
    ncores = os.cpu_count()
    # W untimed and K timed repetitions of the whole workload (about a second
    # each on the host's cores), at most 3 and 20 so the run stays within
    # minutes; the line reports the counts run
    warm, steps = min(max(args.warmup, 0), 3), min(max(args.steps, 1), 20)
    osp = oracle_space(m)
    if warm:
        cpu_assembly(m, kappa, reps=warm, threads=ncores, space=osp)
    nnz, times, used, _ = cpu_assembly(m, kappa, reps=steps, threads=ncores, space=osp)
    t = sum(times) / len(times)
    v = nnz / t
    line = {"metric": METRIC, "value": v, "unit": "nnz/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": len(times), "warmup": warm, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": wl_config(n, {"nnz": int(nnz)}),
            "cpu_baseline": {"value": v, "unit": "nnz/s", "cores": used, "kind": "port",
                             "sample": f"full workload, mean of {len(times)} timed repetitions after {warm} "
                                       f"untimed (OpenMP {used} threads)"},
            "e2e": {"value": v, "unit": "nnz/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "C restatement of GalerkinToolkit's assembly (counting pass, COO append, COO->CSC); "
                    "the Julia reference cannot be installed offline"}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload != "tets":
        {"elasticity": run_elasticity, "batched": run_batched, "serving": run_serving}[args.workload](args)
        return
    import torch
    rep = Replicas("nccl")
    world, rank, local = rep.world, rep.rank, rep.local
    torch.cuda.set_device(local)
    import gtgpu as GT

    n = args.cells
    m, kappa = workload(n)
    ctx = GT.Context(local)
    # one stream for torch and the library: the CUDA events below bracket
    # exactly the library's work.  Above the default priority, like the
    # library's own main stream, so that the element kernels the library
    # queues on its lowest-priority stream fill the gaps of the sparsity
    # kernels instead of holding the SMs ahead of them
    stream = torch.cuda.Stream(priority=-1)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    V = GT.lagrange_space(GT.interior(m), 1, dirichlet_boundary=GT.boundary(m), ctx=ctx)
    kd = torch.from_numpy(kappa).cuda()
    flush = L2Flush()
    a, l = GT.laplacian(kd), GT.source(1.0)

    def step(T=np.float64):
        A, b = GT.assemble_matrix_and_vector(a, l, T, V, out=bdev)
        return A

    bdev = torch.empty(V.num_free_dofs, dtype=torch.float64, device="cuda")
    for _ in range(args.warmup):
        A = step()
        del A
    torch.cuda.synchronize()
    nnz = None
    times = []
    launches0 = ctx.launches()
    rep.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            flush()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            A = step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            nnz = A.nnz
            del A
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    rep.barrier()
    launches = ctx.launches() - launches0
    ms = sum(times) / len(times)
    ms_max = rep.max_ms(ms, "cuda")
    value = rep.value(nnz, ms_max)

    # ---- phase profile of one extra step (dominant kernel + roofline)
    flush()
    ctx.profile_begin()
    A = step()
    phases = ctx.profile_end()
    # the step's CSR and load vector (bitwise those of every timed step) for
    # the parity check against the oracle
    g_rp, g_ci, g_v = A.csr()
    g_b = bdev.cpu().numpy()
    # the captured DRAM traffic belongs to the default workload only
    traffic = TRAFFIC if n == 96 else {}
    spmv = spmv_roofline(A, flush, stream, traffic.get("spmv"))
    del A
    peaks, peaks_kind = load_peaks()
    spmv["frac"] = spmv["achieved"] / peaks["hbm_gbs"]
    spmv["peak"] = peaks["hbm_gbs"]
    fp64_tf = ctx.fma_rate(fp64=True)
    nc, nn = m.num_cells, 4
    nfree = V.num_free_dofs
    ph = {k: v for k, v in phases}
    # algorithmic bytes per launch of the phases
    alg = {
        # reads + Ke/be writes (Ke: the 10 entries of the packed symmetric 4 x 4 block)
        "elements": nc * (4 * 4 + 8) + m.num_nodes * 24 + nc * 10 * 8 + nc * 4 * 8,
        # Ke, be, incidences, cell dofs, rowptr, colind + values, load vector
        "scatter": nc * 10 * 8 + nc * 4 * 8 + nc * 4 * 4 + nc * 4 * 4 + nfree * 8 + nnz * (4 + 8) + nfree * 8,
    }
    # FP64 flops per P1 tetrahedron (FMA = 2, the division = 1): J 9, cofactors
    # 27, det 5, scale 2, six vertex-1..3 entries 36, vertex-0 entries 8, load 6
    flops_el = nc * 93.0
    dom = max((k for k in ph if k in ("elements", "scatter", "pattern_count", "pattern_fill", "incidence")),
              key=lambda k: ph[k])
    # B_asm: the per-matrix algorithmic bytes of the assembly (CSR values
    # written once, cell DOFs, node coordinates once per node, the per-cell
    # coefficient); element matrices are not counted (they would stay on chip)
    b_asm = nnz * 8 + nc * 4 * 4 + m.num_nodes * 24 + nc * 8
    hbm = {}
    for k in ("scatter", "elements"):
        if k in ph:
            gbs = alg[k] / (ph[k] * 1e-3) / 1e9
            hbm[k] = {"achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": gbs / peaks["hbm_gbs"],
                      "algorithmic_bytes": alg[k], "ms": ph[k], "traffic": traffic.get(k),
                      "bytes_counted": "this kernel's reads and writes, the materialised element matrices included"}
    if "scatter" in ph:
        g = b_asm / (ph["scatter"] * 1e-3) / 1e9
        hbm["scatter"]["b_asm"] = {"algorithmic_bytes": b_asm, "achieved": g, "frac": g / peaks["hbm_gbs"]}
    if "scatter" in ph and "elements" in ph:
        t = ph["scatter"] + ph["elements"]
        g = b_asm / (t * 1e-3) / 1e9
        hbm["elements_plus_scatter_b_asm"] = {"algorithmic_bytes": b_asm, "ms": t, "achieved": g, "unit": "GB/s",
                                              "frac": g / peaks["hbm_gbs"]}
    p1_dfloat = os.environ.get("GTGPU_P1") != "fp64"
    if dom == "elements" and p1_dfloat:
        # double-float element arithmetic on the FP32 pipes: the HBM roofline
        # of the kernel's traffic (coordinates, cells, coefficient in; packed
        # blocks and element vectors out); ncu shows it issue-bound
        achieved = alg["elements"] / (ph[dom] * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": "k_elements_p1_df<Laplacian>", "achieved": achieved, "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks_kind,
                "algorithmic_bytes": alg["elements"], "traffic": traffic.get("elements"),
                "arithmetic": "double-float (FP32 pairs, 48-bit) after FP64 differences x_i - x_0; "
                              f"{flops_el / (ph[dom] * 1e-3) / 1e12:.3f} TFLOP/s of FP64-equivalent work "
                              f"(93 flops/cell) against the FP64 FMA rate {fp64_tf:.3f}",
                "limiter": "instruction issue (ncu, 64^3 x 6: issue 68% active, FP64 pipe 45% -- the nine FP64 "
                           "differences per cell --, DRAM 17%)"}
    elif dom == "elements":
        achieved = flops_el / (ph[dom] * 1e-3) / 1e12
        roof = {"bound": "fp64", "kernel": "k_elements_p1<Laplacian, double>", "achieved": achieved,
                "peak": fp64_tf, "unit": "TFLOP/s", "frac": achieved / fp64_tf,
                "peak_source": "measured FP64 FMA rate of this device (gt_ctx_fma_rate); FP64 units, not tensor",
                "peak_method": "gt_ctx_fma_rate: 8 CTAs/SM x 256 threads, 8 independent FMA chains per thread, "
                               "2048 iterations, CUDA events after a warm-up launch (FMA = 2 flops)",
                "algorithmic_flops": flops_el, "traffic": traffic.get("elements")}
    elif dom == "scatter":
        achieved = alg["scatter"] / (ph[dom] * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": "k_scatter_p1<dfl, dfl>" if p1_dfloat else "k_scatter_p1<double, double>",
                "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                "peak_source": peaks_kind, "algorithmic_bytes": alg["scatter"], "traffic": traffic.get("scatter"),
                "b_asm": hbm["scatter"]["b_asm"],
                "limiter": "gathers and the L1 data pipe (ncu, 64^3 x 6: LSU wavefronts 70% of peak -- the column "
                           "searches and row accumulators in shared memory, the gathers --, issue 58%, long_scoreboard "
                           "stalls first, DRAM 32%)"}
    else:
        bytes_dom = alg.get(dom, nnz * 12)
        achieved = bytes_dom / (ph[dom] * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks_kind, "traffic": traffic.get(dom)}
    step_roof = {"algorithmic_bytes": b_asm, "GB/s": b_asm / (ms * 1e-3) / 1e9,
                 "frac_of_hbm": b_asm / (ms * 1e-3) / 1e9 / peaks["hbm_gbs"]}

    # ---- e2e through the C ABI with host buffers
    coords_h = torch.from_numpy(m.coords).pin_memory()
    kappa_h = torch.from_numpy(kappa).pin_memory()
    rp_h = torch.empty(nfree + 1, dtype=torch.int64).pin_memory()
    ci_h = torch.empty(nnz, dtype=torch.int32).pin_memory()
    v_h = torch.empty(nnz, dtype=torch.float64).pin_memory()
    b_h = torch.empty(nfree, dtype=torch.float64).pin_memory()
    from gtgpu.api import _ptr
    import ctypes as C
    lib = ctx.lib
    f_one = np.ones(1)
    e2e_times = []
    for it in range(args.warmup + max(3, args.steps // 2)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        # coordinates and coefficient in, CSR + load vector out, in the one
        # reference-facing call (uploads and the pattern download overlap the
        # kernels on the library's copy stream)
        V.dmesh.set_coords(coords_h)
        h = C.c_void_p()
        GT.api.check(ctx.h, lib.gt_assemble_csr(V.h, GT.api._lib.GT_LAPLACE, _ptr(kappa_h), 0.3, GT.api._lib.GT_FP64,
                                                _ptr(f_one), None, _ptr(b_h), nnz, _ptr(rp_h), _ptr(ci_h),
                                                _ptr(v_h), None, C.byref(h)))
        lib.gt_matrix_destroy(h)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            e2e_times.append(dt)
    e2e_ms = 1e3 * sum(e2e_times) / len(e2e_times)
    h2d = m.coords.nbytes + kappa.nbytes
    d2h = rp_h.numel() * 8 + nnz * 4 + nnz * 8 + nfree * 8

    # ---- solve: plain FP64 PCG vs FP32 PCG with FP64 reliable updates,
    # latency over SOLVE_SAMPLES timed solves each
    solve = None
    xs = {}
    if not args.no_solve:
        Am, bm = GT.assemble_matrix_and_vector(a, l, "mixed", V)
        res = {}
        for mode in ("fp64", "ir"):
            lat = []
            GT.solve(Am, bm, rtol=SOLVE_RTOL, mode=mode)  # warm-up (sliced-ELL copy, graphs)
            for r in range(SOLVE_SAMPLES):
                t0 = time.perf_counter()
                x, info = GT.solve(Am, bm, rtol=SOLVE_RTOL, mode=mode)
                lat.append(time.perf_counter() - t0)
            xs[mode] = x
            lat = np.array(lat)
            res[mode] = {"solves_per_s": 1.0 / float(lat.mean()), "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                         "p99_ms": 1e3 * float(np.percentile(lat, 99)), "samples": int(lat.size),
                         "iterations": info["iterations"], "fp64_iterations": info["fp64_iterations"],
                         "true_residual_updates": info["outer_iterations"], "rel_residual": info["rel_residual"],
                         "ms_per_iteration": 1e3 * float(lat.min()) / max(1, info["iterations"])}
        res["ir_vs_fp64_rel_err"] = _relerr(xs["ir"], xs["fp64"])
        res["mixed_vs_fp64_speedup"] = res["ir"]["solves_per_s"] / res["fp64"]["solves_per_s"]
        res["rtol"] = SOLVE_RTOL
        solve = res
        del Am

    # ---- CPU: the oracle (C restatement of the reference) on the same
    # workload, single-threaded like the reference and on all host cores;
    # its CSR, load vector and FP64 solution are the parity references
    cpu, parity = None, None
    if rank == 0 and not args.no_cpu:
        O = _oracle()
        osp = oracle_space(m)
        cnnz, t1, _, _ = cpu_assembly(m, kappa, reps=1, threads=1, space=osp)
        ncores = os.cpu_count()
        cnnz, tn, used, (cp, rv, nz, ob) = cpu_assembly(m, kappa, reps=1, threads=ncores, space=osp)
        orp, oci, ov = O.csc_to_csr(cp, rv, nz, osp["nfree"])
        t0 = time.perf_counter()
        _, cg_it, cg_rr = O.pcg(orp, oci, ov, ob, rtol=SOLVE_RTOL)
        cg_s = time.perf_counter() - t0
        cpu = {"value": cnnz / min(tn), "unit": "nnz/s", "cores": used, "kind": "port",
               "sample": f"full workload, 1 repetition (C restatement of the reference, OpenMP {used} threads)",
               "single_thread": {"value": cnnz / min(t1), "unit": "nnz/s", "cores": 1, "seconds": min(t1),
                                 "sample": "full workload, 1 repetition, 1 thread (the reference is single-threaded)"},
               "solve": {"seconds": cg_s, "solves_per_s": 1.0 / cg_s, "iterations": cg_it, "rel_residual": cg_rr,
                         "rtol": SOLVE_RTOL, "threads": 1,
                         "kind": "oracle FP64 Jacobi-PCG on the oracle's CSR (the reference solves with a direct "
                                 "LU; it has no CG)"}}
        parity = {"oracle": "oracle/gt_oracle.c (C restatement of the reference), same seeded mesh and kappa",
                  "pattern_equal": bool(np.array_equal(g_rp, orp) and np.array_equal(g_ci, oci)),
                  "values_max_rel_err": _relerr(g_v, ov) if g_v.size == ov.size else None,
                  "load_vector_max_rel_err": _relerr(g_b, ob),
                  "tolerance": {"values": 1e-12, "load_vector": 1e-12, "solution": 1e-8},
                  "error_scale": "max |gpu - oracle| / max |oracle|"}
        if xs:
            xo, o_it, o_rr = O.pcg(orp, oci, ov, ob, rtol=1e-12)
            parity["solution_ref"] = f"oracle FP64 PCG to rel. residual {o_rr:.1e} ({o_it} iterations)"
            parity["solution_max_rel_err"] = {k: _relerr(v, xo) for k, v in xs.items()}

    line = {"metric": METRIC, "value": value, "unit": "nnz/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": wl_config(n, {"nnz": int(nnz), "free_dofs": int(nfree), "parallelism": f"replicas x{world}"}),
            "e2e": {"value": rep.value(nnz, rep.max_ms(e2e_ms, "cuda")), "unit": "nnz/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "resident": "the space (cell DOF ids, free-first numbering) stays on the device; coordinates "
                                "and kappa are uploaded and the CSR + load vector downloaded every step"},
            "roofline": roof, "step_roofline": step_roof, "hbm_kernels": {**hbm, "spmv_fp64": spmv},
            "phases_ms": {k: round(v, 4) for k, v in phases},
            "cpu_baseline": cpu, "parity": parity, "solve": solve, "clocks": clocks.summary(),
            "gpu_launches": int(launches), "wall_s_timed": t_wall}
    if rank == 0:
        print(json.dumps(line), flush=True)
    rep.close()


if __name__ == "__main__":
    main()
