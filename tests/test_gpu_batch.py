"""Batched solves through the C ABI: every instance's batched solution
matches its stand-alone solve, and an instance's result is bitwise the same
alone and inside the batch."""
import numpy as np
import pytest

import gtgpu as GT
from gtgpu import batch as GB

pytestmark = pytest.mark.gpu


def _instances():
    specs = [GB.InstanceSpec(0, 2, 1, 9), GB.InstanceSpec(1, 2, 2, 6), GB.InstanceSpec(2, 3, 1, 5),
             GB.InstanceSpec(3, 3, 2, 3), GB.InstanceSpec(4, 2, 1, 31), GB.InstanceSpec(5, 3, 1, 7),
             GB.InstanceSpec(6, 2, 2, 2), GB.InstanceSpec(7, 3, 2, 4)]
    return [GB.assemble_instance(s, seed=7, T="mixed") for s in specs]


@pytest.mark.parametrize("mode", ["fp64", "ir"])
def test_batch_matches_single_solves(mode):
    inst = _instances()
    mats = [A for _, _, A, _ in inst]
    bs = [b for _, _, _, b in inst]
    B = GB.Batch(mats)
    x, infos = B.solve(bs, rtol=1e-10, mode=mode)
    for (m, V, A, b), xi, info in zip(inst, B.split(x), infos):
        xs, _ = GT.solve(A, b, rtol=1e-12, mode="fp64")
        assert info["rel_residual"] <= 1e-10
        assert np.abs(xi - xs).max() <= 1e-8 * max(np.abs(xs).max(), 1e-300)


def test_batch_result_independent_of_batch_mix():
    inst = _instances()
    mats = [A for _, _, A, _ in inst]
    bs = [b for _, _, _, b in inst]
    full, _ = GB.Batch(mats).solve(bs, rtol=1e-8, mode="ir")
    xs_full = GB.Batch(mats).split(full)
    for k in (1, 3, 5):
        alone, _ = GB.Batch([mats[k]]).solve([bs[k]], rtol=1e-8, mode="ir")
        assert np.array_equal(alone, xs_full[k])


def _elasticity_instances(T="mixed"):
    """3-D linear elasticity (block size 3) on Q1 and Q2 hexahedra, clamped
    at x = 0, lognormal(0, 0.5) Young's modulus per cell"""
    out = []
    for k, (order, n) in enumerate([(1, 4), (2, 3), (1, 6), (2, 2)]):
        m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (n, n, n))
        coef = GT.lognormal_cells(m.num_cells, 0.5, 900 + k)
        V = GT.lagrange_space(GT.interior(m), order, tensor_size=(3,), dirichlet_boundary=GT.boundary(m, ["2-face-5"]))
        A, b = GT.assemble_matrix_and_vector(GT.elasticity(coef, 0.3), GT.source([0.0, 0.0, -1.0]), T, V)
        out.append((m, V, A, b))
    return out


@pytest.mark.parametrize("mode", ["fp64", "ir"])
def test_batch_of_block_matrices(mode):
    """Elasticity (3 x 3 blocks) and scalar instances in one batch: one launch
    per block size; every solution within 1e-8 of its stand-alone FP64 solve
    and bitwise the same alone and in the mix."""
    el = _elasticity_instances()
    sc = _instances()[:3]
    mats = [A for _, _, A, _ in el] + [A for _, _, A, _ in sc]
    bs = [b for _, _, _, b in el] + [b for _, _, _, b in sc]
    B = GB.Batch(mats)
    assert B.info()["small_instances"] == len(mats)
    x, infos = B.solve(bs, rtol=1e-10, mode=mode)
    parts = B.split(x)
    for k, (A, b) in enumerate(zip(mats, bs)):
        xs, _ = GT.solve(A, b, rtol=1e-12, mode="fp64")
        assert infos[k]["rel_residual"] <= 1e-10
        assert np.abs(parts[k] - xs).max() <= 1e-8 * np.abs(xs).max()
    for k in (0, 1, 4):
        alone, _ = GB.Batch([mats[k]]).solve([bs[k]], rtol=1e-10, mode=mode)
        assert np.array_equal(alone, parts[k])


@pytest.mark.parametrize("mode", ["fp64", "ir"])
def test_grouped_tier_is_bitwise_the_single_solves(mode):
    """Medium instances (above the one-CTA limit, up to 262,144 rows) share
    grouped persistent launches, each on the CTAs of its own solve: every
    solution is bitwise what gt_solve gives for the instance alone, scalar
    and 3 x 3 block matrices alike."""
    specs = [GB.InstanceSpec(0, 2, 1, 150), GB.InstanceSpec(1, 3, 1, 30), GB.InstanceSpec(2, 2, 2, 60),
             GB.InstanceSpec(3, 2, 1, 9), GB.InstanceSpec(4, 3, 2, 12)]
    inst = [GB.assemble_instance(s, seed=8, T="mixed") for s in specs]
    m = GT.cartesian_mesh((0, 1, 0, 1, 0, 1), (12, 12, 12))
    V = GT.lagrange_space(GT.interior(m), 1, tensor_size=(3,), dirichlet_boundary=GT.boundary(m, ["2-face-5"]))
    Ae, be = GT.assemble_matrix_and_vector(GT.elasticity(GT.lognormal_cells(m.num_cells, 0.5, 77), 0.3),
                                           GT.source([0.0, 0.0, -1.0]), "mixed", V)
    mats = [A for _, _, A, _ in inst] + [Ae]
    bs = [b for _, _, _, b in inst] + [be]
    B = GB.Batch(mats, small_rows=1024)
    assert B.info()["small_instances"] == 1
    x, infos = B.solve(bs, rtol=1e-10, mode=mode)
    for k, (A, b, xb) in enumerate(zip(mats, bs, B.split(x))):
        xs, info = GT.solve(A, b, rtol=1e-10, mode=mode)
        assert infos[k]["rel_residual"] <= 1e-10
        if A.shape[0] > 1024:
            assert np.array_equal(xb, xs), k
            assert infos[k]["iterations"] == info["iterations"]


def test_autotune_picks_a_candidate(tmp_path):
    inst = _instances()
    B = GB.Batch([A for _, _, A, _ in inst])
    b = np.concatenate([b for _, _, _, b in inst])
    entry = GB.autotune_lanes(B, b, iters=16, cache=str(tmp_path / "tune.json"))
    assert entry["lanes"] in (1, 2, 4, 8)
    assert B.info()["lanes"] == entry["lanes"]
    again = GB.autotune_lanes(B, b, cache=str(tmp_path / "tune.json"))
    assert again["lanes"] == entry["lanes"]


def test_autotune_batch_picks_workers_tier_and_lanes(tmp_path):
    """autotune_batch times run_batch per worker count and per row limit of
    the one-CTA tier on a sample, tunes the lanes, and caches the choice."""
    specs = [GB.InstanceSpec(i, 2 + (i % 2), 1 + (i // 2) % 2, n) for i, n in enumerate((9, 5, 40, 7, 70, 4, 24, 6))]
    inputs = {s.index: GB.instance_inputs(s, seed=5) for s in specs}
    cache = str(tmp_path / "tune.json")
    e = GB.autotune_batch(specs, inputs, "mixed", rtol=1e-8, workers=(1, 2), small_rows=(1024, 32768), cache=cache)
    assert e["workers"] in (1, 2) and e["small_rows"] in (1024, 32768) and e["lanes"] in (0, 1, 2, 4, 8)
    assert set(e["small_rows_seconds"]) == {"1024", "32768"}
    assert GB.autotune_batch(specs, inputs, "mixed", rtol=1e-8, cache=cache) == e
    r = GB.run_batch(specs, inputs, "mixed", rtol=1e-8, workers=e["workers"], small_rows=e["small_rows"],
                     lanes=e["lanes"] or None)
    assert all(i["rel_residual"] <= 1e-8 for i in r.infos.values())


def test_batch_with_large_instance_matches_alone():
    """A batch mixing one-CTA instances with one above the size limit (solved
    by the persistent grid solver): every result equals its solve alone."""
    specs = [GB.InstanceSpec(0, 2, 1, 200), GB.InstanceSpec(1, 2, 1, 9), GB.InstanceSpec(2, 3, 2, 3)]
    inst = [GB.assemble_instance(s, seed=11, T="mixed") for s in specs]
    mats = [A for _, _, A, _ in inst]
    bs = [b for _, _, _, b in inst]
    B = GB.Batch(mats)
    assert B.info()["small_instances"] == 2
    for mode in ("fp64", "ir"):
        x, infos = B.solve(bs, rtol=1e-9, mode=mode)
        parts = B.split(x)
        for k in range(3):
            assert infos[k]["rel_residual"] <= 1e-9
            alone, _ = GB.Batch([mats[k]]).solve([bs[k]], rtol=1e-9, mode=mode)
            assert np.array_equal(alone, parts[k])


def test_run_batch_concurrent_workers_bitwise_and_converged():
    """run_batch with several worker contexts (concurrent assembly, large
    instances solved on the workers' streams, the small ones in one launch)
    gives bitwise the results of one worker, in mixed and plain FP64."""
    specs = [GB.InstanceSpec(0, 2, 1, 9), GB.InstanceSpec(1, 2, 2, 30), GB.InstanceSpec(2, 3, 1, 12),
             GB.InstanceSpec(3, 3, 2, 5), GB.InstanceSpec(4, 2, 1, 120), GB.InstanceSpec(5, 3, 1, 7),
             GB.InstanceSpec(6, 2, 2, 3), GB.InstanceSpec(7, 3, 2, 9)]
    inputs = {s.index: GB.instance_inputs(s, seed=21) for s in specs}
    for prec in ("mixed", "fp64"):
        one = GB.run_batch(specs, inputs, prec, rtol=1e-10, workers=1, small_rows=2000)
        three = GB.run_batch(specs, inputs, prec, rtol=1e-10, workers=3, small_rows=2000)
        assert one.small + one.large == len(specs) and one.large >= 3 and one.small >= 3
        for s in specs:
            assert three.infos[s.index]["rel_residual"] <= 1e-10
            assert np.array_equal(one.solutions[s.index], three.solutions[s.index])
