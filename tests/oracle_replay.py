"""The adjoint's forward map restated on the CPU oracle (test infrastructure).

samurai has no derivatives: the GPU adjoint (sg_adjoint_*) differentiates the
time loop of demos/FiniteVolume/advection_2d.cpp:140-147 on the mesh sequence
that its forward pass recorded.  These helpers give the same two maps with the
oracle, so that the GPU adjoint is checked against the reference operator and
not against itself:

* record(): the loop with adaptation (Adapt::harten pass by pass,
  mr/adapt.hpp:147-195, then update_ghost_mr and the upwind step), keeping the
  leaf cells after every Harten pass that changed the mesh;
* replay(): the recorded steps on the recorded meshes from other initial
  values: per transition the ghost update then update_fields onto the next
  recorded mesh (mr/adapt.hpp:380-386, algorithm/update_fields.hpp:27-127),
  then the ghost update and the upwind step (stencil_field.hpp:38-97).

Both run in worker processes started with `spawn` when several are wanted at
once (finite differences), so that no worker is forked from a process that
already holds a CUDA context.
"""
import multiprocessing as mp
import os
import shutil
import tempfile

import numpy as np

from oracle.pyoracle import OracleSim


def record(dim, minl, maxl, cells0, u0, n_steps, eps, regularity, a, dt, scheme=0):
    """(steps, final): steps[n] lists the leaf meshes (level, coords) that step
    n's Harten passes produced; final = (level, coords, uT)."""
    o = OracleSim(dim, minl, maxl, 1, 1)
    o.set_cells(*cells0)
    o.set_cell_values(u0)
    steps = []
    for _ in range(n_steps):
        trans = []
        for i in range(maxl - minl):
            if o.harten(i, eps, regularity):
                break
            lv, co, _ = o.cells()
            trans.append((lv, co))
        steps.append(trans)
        o.update_ghost()
        o.upwind(list(a), dt, scheme)
    lv, co, _ = o.cells()
    return steps, (lv, co, o.cell_values())


def replay(dim, minl, maxl, cells0, steps, u0, a, dt, scheme=0):
    """uT of the recorded steps on the recorded meshes from leaf values u0"""
    o = OracleSim(dim, minl, maxl, 1, 1)
    o.set_cells(*cells0)
    o.set_cell_values(u0)
    for trans in steps:
        for lv, co in trans:
            o.update_ghost()
            o.transfer_cells(lv, co)
        o.update_ghost()
        o.upwind(list(a), dt, scheme)
    return o.cell_values()


_STATE = {}


def save_sequence(path, cells0, steps):
    """the initial mesh and the recorded mesh sequence in one .npz file"""
    meshes = [cells0] + [m for trans in steps for m in trans]
    np.savez(path, level=np.concatenate([m[0] for m in meshes]).astype(np.int8),
             coords=np.concatenate([m[1] for m in meshes]).astype(np.int32),
             counts=np.array([len(m[0]) for m in meshes], np.int64), per_step=np.array([len(t) for t in steps], np.int64))


def load_sequence(path):
    # each member of the archive is read once (indexing an NpzFile reads the member from the file again)
    with np.load(path) as f:
        level, coords, counts, per_step = f["level"], f["coords"], f["counts"], f["per_step"]
    ends = np.cumsum(counts)
    meshes = [(level[e - n:e], coords[e - n:e]) for n, e in zip(counts, ends)]
    steps, k = [], 1
    for n in per_step:
        steps.append(meshes[k:k + n])
        k += int(n)
    return meshes[0], steps


def _init(dim, minl, maxl, path, dt, scheme):
    cells0, steps = load_sequence(path)
    _STATE.update(dim=dim, minl=minl, maxl=maxl, cells0=cells0, steps=steps, dt=dt, scheme=scheme)


def _job(args):
    u0, a = args
    s = _STATE
    return replay(s["dim"], s["minl"], s["maxl"], s["cells0"], s["steps"], u0, a, s["dt"], s["scheme"])


class ReplayPool:
    """replay() of many (u0, a) pairs on a pool of spawned worker processes;
    the workers read the mesh sequence from a file rather than each receiving
    a pickled copy"""

    def __init__(self, processes, dim, minl, maxl, cells0, steps, dt, scheme=0):
        self.dir = tempfile.mkdtemp(prefix="oracle_replay_")
        self.path = os.path.join(self.dir, "sequence.npz")
        save_sequence(self.path, cells0, steps)
        ctx = mp.get_context("spawn")
        self.pool = ctx.Pool(processes, initializer=_init, initargs=(dim, minl, maxl, self.path, dt, scheme))

    def map(self, jobs):
        return self.pool.map(_job, [(np.ascontiguousarray(u, np.float64), tuple(a)) for u, a in jobs])

    def close(self):
        self.pool.close()
        self.pool.join()
        shutil.rmtree(self.dir, ignore_errors=True)
