"""The N > 1 layout of the benchmark on CPU: two `gloo` ranks run the
replica helper of bench.py (barriers, max over ranks of the step time,
whole-job throughput), build the same seeded workload mesh, and only rank 0
of the reference arm does work or prints.  No GPU is used."""
import contextlib
import hashlib
import io
import os
import socket
import sys
import types

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch
    import bench
    rep = bench.Replicas("gloo")
    assert (rep.world, rep.rank, rep.local) == (world, rank, rank)
    rep.barrier()
    # rank r took 1 + r ms per step: every rank sees the slowest
    ms = rep.max_ms(1.0 + rank, "cpu")
    value = rep.value(1000, ms)
    # every replica assembles the same seeded workload (weak scaling: the
    # per-rank work is fixed); compare a digest of the mesh across ranks
    m, kappa = bench.workload(3)
    h = hashlib.sha256()
    for a in (m.coords, m.cell_nodes, kappa):
        h.update(np.ascontiguousarray(a).tobytes())
    d = torch.tensor(list(h.digest()[:8]), dtype=torch.int64)
    ds = [torch.zeros_like(d) for _ in range(world)]
    rep.dist.all_gather(ds, d)
    same = all(bool((x == ds[0]).all()) for x in ds)
    # the reference arm: ranks other than 0 exit without work or output
    buf = io.StringIO()
    if rank != 0:
        with contextlib.redirect_stdout(buf):
            bench.run_reference(types.SimpleNamespace(cells=96, warmup=3, steps=10, gpus=world))
    rep.barrier()
    rep.close()
    with open(os.path.join(outdir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{ms} {value} {int(same)} {len(buf.getvalue())}\n")


@pytest.mark.timeout(300)
def test_two_gloo_replicas(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    for r in range(world):
        ms, value, same, out = open(tmp_path / f"rank{r}.txt").read().split()
        assert float(ms) == 2.0
        assert float(value) == pytest.approx(world * 1000 / 2e-3)
        assert same == "1"
        assert out == "0"


def test_single_process_replica_has_no_collectives(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    rep = bench.Replicas("gloo")
    assert (rep.world, rep.rank, rep.local) == (1, 0, 0)
    rep.barrier()
    assert rep.max_ms(3.5, "cpu") == 3.5
    assert rep.value(7, 2.0) == pytest.approx(3500.0)
    rep.close()
