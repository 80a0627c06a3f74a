"""One instance of the batched workload stepped by the CPU oracle (test
infrastructure), for the batched-mode parity test.  run_instance() takes the
seed, the instance count and the instance's position (the instance's initial
condition is a closure that a spawned worker regenerates), so that the
instances run in parallel on a pool of processes started with `spawn`."""
from advection_cases import batch_instances
from oracle.pyoracle import MESH_IDS, OracleSim


def run_instance(args):
    """(cells, values, intervals) of instance k after the initial adaptation
    and `steps` steps of adapt, update_ghost_mr and upwind (the calls of the
    demo's time loop, demos/FiniteVolume/advection_2d.cpp:140-147)"""
    seed, n, k, steps = args
    p = batch_instances(seed, n)[k]
    o = OracleSim(2, p["min_level"], p["max_level"], 1, 1)
    lv, co, _ = o.cells()
    o.set_cell_values(p["u0"](lv, co))
    passes = [o.adapt(p["eps"], p["regularity"])]
    for _ in range(steps):
        passes.append(o.adapt(p["eps"], p["regularity"]))
        o.update_ghost()
        o.upwind(list(p["a"]), p["dt"], 0)
    ivs = {(mid, lev): o.intervals(mid, lev) for mid in MESH_IDS for lev in range(p["max_level"] + 1)}
    return o.cells(), o.cell_values(), ivs, passes
