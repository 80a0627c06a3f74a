"""Batched mode (sg_batch_*): independent problems advanced together must give,
instance by instance, exactly what the serial calls give (meshes identical,
FP64 fields bit-identical), and the serial calls match the oracle."""
import multiprocessing as mp
import os

import numpy as np
import pytest

from advection_cases import ball_3d, batch_instances
from gpu_util import compare_cells, compare_fields, compare_meshes
from oracle.pyoracle import OracleSim

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from samurai_gb300 import build

    build.build()
    import samurai_gb300

    return samurai_gb300


def make_problems(sg, seed, n, with_3d):
    probs = batch_instances(seed, n, max_levels=(5, 8))
    if with_3d:
        probs.append(dict(min_level=2, max_level=5, a=(1.0, 0.75, -0.5), eps=1e-3, regularity=1.0, dt=0.3 / 32, u0=ball_3d(5), dim=3))
    sims = []
    for p in probs:
        dim = p.get("dim", 2)
        s = sg.AdvectionSim(dim, p["min_level"], p["max_level"])
        lv, co, _ = s.cells()
        s.set_cell_values(p["u0"](lv, co))
        sims.append(s)
    return probs, sims


def same_state(a, b, max_level, where):
    lg, cg, ig = a.cells()
    ls, cs, is_ = b.cells()
    assert np.array_equal(lg, ls) and np.array_equal(cg, cs) and np.array_equal(ig, is_), where + ": leaf cells differ"
    for mid in ("cells", "reference"):
        for level in range(max_level + 1):
            assert np.array_equal(a.intervals(mid, level), b.intervals(mid, level)), "%s: %s level %d" % (where, mid, level)
    va, vb = a.cell_values(), b.cell_values()
    bad = np.flatnonzero(va != vb)
    assert bad.size == 0, "%s: %d leaf values differ" % (where, bad.size)


def test_batch_autotune_keeps_state_and_results(sg):
    """sg_batch_autotune leaves every instance as it found it, and the
    batch stepped under the chosen shape still matches the serial calls"""
    probs, batched = make_problems(sg, 13, 6, with_3d=False)
    _, serial = make_problems(sg, 13, 6, with_3d=False)
    batch = sg.Batch(batched, n_threads=2)
    eps = [p["eps"] for p in probs]
    reg = [p["regularity"] for p in probs]
    a = [p["a"] for p in probs]
    dt = [p["dt"] for p in probs]
    batch.adapt(eps, reg)
    for p, s in zip(probs, serial):
        s.adapt(p["eps"], p["regularity"])
    batch.synchronize()
    before = [(s.cells(), s.cell_values()) for s in batched]
    d_ms, t_ms, shape = batch.autotune(eps, reg, a, dt, steps=2)
    assert 0 < t_ms <= d_ms
    assert shape["fuse_words"] in (0, 128, 1024, 10000, 100000) and shape["block"] in (0, 128, 256, 512)
    for k, s in enumerate(batched):
        (lv, co, ix), vals = s.cells(), s.cell_values()
        assert np.array_equal(lv, before[k][0][0]) and np.array_equal(co, before[k][0][1]), "instance %d: cells changed" % k
        assert np.array_equal(vals, before[k][1]), "instance %d: values changed" % k
    for step in range(3):
        batch.step(eps, reg, a, dt)
        for p, s in zip(probs, serial):
            s.adapt(p["eps"], p["regularity"])
            s.update_ghost()
            s.upwind(p["a"], p["dt"])
        batch.synchronize()
        for k, (p, s) in enumerate(zip(probs, serial)):
            same_state(batched[k], s, p["max_level"], "tuned step %d, instance %d" % (step, k))
    batch.close()


@pytest.mark.parametrize("n_threads", [1, 4])
def test_batch_matches_serial(sg, n_threads):
    probs, batched = make_problems(sg, 11, 9, with_3d=True)
    _, serial = make_problems(sg, 11, 9, with_3d=True)
    batch = sg.Batch(batched, n_threads=n_threads)
    eps = [p["eps"] for p in probs]
    reg = [p["regularity"] for p in probs]
    a = [p["a"] for p in probs]
    dt = [p["dt"] for p in probs]

    # initial adaptation through the split calls
    passes = batch.adapt(eps, reg)
    for k, (p, s) in enumerate(zip(probs, serial)):
        assert s.adapt(p["eps"], p["regularity"]) == passes[k]
        same_state(batched[k], s, p["max_level"], "initial adaptation, instance %d" % k)

    for step in range(6):
        passes = batch.step(eps, reg, a, dt).copy()
        for k, (p, s) in enumerate(zip(probs, serial)):
            assert s.adapt(p["eps"], p["regularity"]) == passes[k]
            s.update_ghost()
            s.upwind(p["a"], p["dt"])
        batch.synchronize()
        for k, (p, s) in enumerate(zip(probs, serial)):
            same_state(batched[k], s, p["max_level"], "step %d, instance %d" % (step, k))
    batch.close()


def test_batch_instance_matches_oracle(sg):
    probs, sims = make_problems(sg, 23, 4, with_3d=False)
    batch = sg.Batch(sims, n_threads=2)
    oras = []
    for p in probs:
        o = OracleSim(2, p["min_level"], p["max_level"], 1, 1)
        lv, co, _ = o.cells()
        o.set_cell_values(p["u0"](lv, co))
        o.adapt(p["eps"], p["regularity"])
        oras.append(o)
    batch.adapt([p["eps"] for p in probs], [p["regularity"] for p in probs])
    for step in range(3):
        batch.step([p["eps"] for p in probs], [p["regularity"] for p in probs], [p["a"] for p in probs], [p["dt"] for p in probs])
        for p, o in zip(probs, oras):
            o.adapt(p["eps"], p["regularity"])
            o.update_ghost()
            o.upwind(p["a"], p["dt"])
    for k, (p, g, o) in enumerate(zip(probs, sims, oras)):
        compare_meshes(g, o, p["max_level"], "instance %d" % k)
        compare_cells(g, o, "instance %d" % k)
        compare_fields(g, o, "instance %d" % k, cells_only=True)
    batch.close()


def test_batch_rejects_shared_mesh(sg):
    s = sg.AdvectionSim(2, 2, 5)
    with pytest.raises(sg.SamuraiGpuError, match="share a mesh"):
        sg.Batch([s, s])


def test_batch_benchmark_instances_against_oracle(sg):
    """18 instances of the benchmark's batched workload (seed 2027: max_level 7
    to 11, both thresholds, max_level 11 with each), through the batched
    calls for the initial adaptation and 3 steps, against the oracle stepping
    each instance alone: every mesh id, the leaf cells and their values, bit
    for bit, and the Harten pass counts."""
    seed, n, steps = 2027, 256, 3
    idx = list(range(16)) + [20, 23]
    probs = batch_instances(seed, n)
    assert {probs[k]["max_level"] for k in idx} == {7, 8, 9, 10, 11}
    assert {probs[k]["eps"] for k in idx if probs[k]["max_level"] == 11} == {1e-3, 1e-4}
    # the oracle runs while the GPU works: spawned workers (no fork after CUDA initialisation)
    pool = mp.get_context("spawn").Pool(min(len(idx), os.cpu_count() or 1))
    from oracle_batch import run_instance

    pending = pool.map_async(run_instance, [(seed, n, k, steps) for k in idx])
    sims = []
    for k in idx:
        p = probs[k]
        s = sg.AdvectionSim(2, p["min_level"], p["max_level"])
        lv, co, _ = s.cells()
        s.set_cell_values(p["u0"](lv, co))
        sims.append(s)
    batch = sg.Batch(sims, n_threads=4)
    eps = [probs[k]["eps"] for k in idx]
    reg = [probs[k]["regularity"] for k in idx]
    passes = [list(batch.adapt(eps, reg))]
    for _ in range(steps):
        passes.append(list(batch.step(eps, reg, [probs[k]["a"] for k in idx], [probs[k]["dt"] for k in idx])))
    batch.synchronize()
    results = pending.get(timeout=1800)
    pool.close()
    pool.join()
    for j, (k, g) in enumerate(zip(idx, sims)):
        (lo, coo, io), vo, ivs, po = results[j]
        where = "instance %d (max_level %d)" % (k, probs[k]["max_level"])
        assert [p[j] for p in passes] == po, where + ": Harten passes"
        lg, cg, ig = g.cells()
        assert np.array_equal(lg, lo) and np.array_equal(cg, coo) and np.array_equal(ig, io), where + ": leaf cells"
        assert np.array_equal(g.cell_values(), vo), where + ": leaf values"
        for (mid, lev), iv in ivs.items():
            assert np.array_equal(g.intervals(mid, lev), iv), "%s: %s level %d" % (where, mid, lev)
    batch.close()
