"""The GPU adjoint against the reference operator, on the differentiation
workload at its full size: 2D, min_level 3, max_level 10, a = (1, 0.7), eps
1e-4, regularity 2, 256 steps, checkpoints every 16 steps, J = sum vol (u_T -
u_tgt)^2 with a seeded Gaussian target.

The oracle restates the forward map (tests/oracle_replay.py): the loop with
adaptation records the mesh sequence, and the frozen-mesh replay reruns the
recorded steps on it.  Checked here:

* the GPU's recorded forward (sg_adjoint_record) is the oracle's loop: the same
  final mesh and the same values, bit for bit;
* the GPU's frozen-mesh replay (sg_adjoint_replay) is the oracle's replay, bit
  for bit, from the recorded u0 and from a random field;
* dot-product test against the oracle: <L v, w> with L v from the oracle's
  replay equals <v, L^T w> with L^T w from the GPU's backward pass;
* central finite differences of J through the oracle's replay along 8 seeded
  directions in u0 (h = 1e-3: J is quadratic in u0 on a frozen mesh, so the
  difference quotient is exact up to rounding) and along both velocity
  components (h = 1e-6), against the GPU's dJ/du0 and dJ/da: relative error
  at most 1e-6, the tolerance of the adjoint's specification.

The oracle's replays run in parallel on spawned worker processes."""
import os

import numpy as np
import pytest

import oracle_replay as orp
from advection_cases import cell_volumes, gaussian_target, shapes_2d
from oracle.pyoracle import OracleSim

pytestmark = pytest.mark.gpu

MINL, MAXL, STEPS, EPS, REG, K = 3, 10, 256, 1e-4, 2.0, 16
A = (1.0, 0.7)
DT = 0.5 / (1 << MAXL)
N_DIRECTIONS = 8


@pytest.fixture(scope="module")
def c4():
    from samurai_gb300 import build

    build.build()
    import samurai_gb300 as sg

    # the same adapted start on both sides
    o = OracleSim(2, MINL, MAXL, 1, 1)
    lv, co, _ = o.cells()
    vals = shapes_2d(2028, 8, 8)(lv, co)
    o.set_cell_values(vals)
    s = sg.AdvectionSim(2, MINL, MAXL)
    s.set_cell_values(vals)
    assert s.adapt(EPS, REG) == o.adapt(EPS, REG)
    lv, co, _ = o.cells()
    lg, cg, _ = s.cells()
    assert np.array_equal(lv, lg) and np.array_equal(co, cg)
    u0 = o.cell_values()
    assert np.array_equal(u0, s.cell_values())
    cells0 = (lv, co)

    # the oracle's loop with adaptation: mesh sequence and final state
    steps, (lvT, coT, uT) = orp.record(2, MINL, MAXL, cells0, u0, STEPS, EPS, REG, A, DT)

    adj = sg.Adjoint(s.u, checkpoint_every=K)
    uT_gpu = adj.record(u0, STEPS, EPS, REG, A, DT)
    lvg, cog = adj.cells("final")
    tgt = gaussian_target(2029)(lvT, coT)
    vol = cell_volumes(lvT)

    def J(u):
        return float(np.sum(vol * (u - tgt) ** 2))

    rng = np.random.default_rng(2030)
    n0, nT = len(u0), len(uT)
    v, w = rng.standard_normal(n0), rng.standard_normal(nT)
    dirs = [rng.standard_normal(n0) for _ in range(N_DIRECTIONS)]
    hu, ha = 1e-3, 1e-6
    jobs = [(u0, A), (v, A)]
    for d in dirs:
        jobs += [(u0 + hu * d, A), (u0 - hu * d, A)]
    for k in range(2):
        ap, am = list(A), list(A)
        ap[k] += ha
        am[k] -= ha
        jobs += [(u0, ap), (u0, am)]
    pool = orp.ReplayPool(min(len(jobs), os.cpu_count() or 1), 2, MINL, MAXL, cells0, steps, DT)
    try:
        out = pool.map(jobs)
    finally:
        pool.close()

    g0, ga = adj.backward(2.0 * vol * (uT_gpu - tgt))
    LTw, _ = adj.backward(w)
    res = dict(adj=adj, u0=u0, v=v, w=w, uT=uT, lvT=lvT, coT=coT, uT_gpu=uT_gpu, lvg=lvg, cog=cog, J=J, g0=g0, ga=ga, LTw=LTw,
               replay_u0=out[0], replay_v=out[1], dirs=dirs, hu=hu, ha=ha, fd_jobs=out[2:])
    yield res
    adj.close()


def test_recorded_forward_is_the_oracle_loop(c4):
    assert np.array_equal(c4["lvg"], c4["lvT"]) and np.array_equal(c4["cog"], c4["coT"]), "final meshes differ"
    assert np.array_equal(c4["uT_gpu"], c4["uT"]), "final values differ"
    # the oracle's replay of its own recording reproduces its loop
    assert np.array_equal(c4["replay_u0"], c4["uT"])


def test_frozen_replay_is_the_oracle_replay(c4):
    adj = c4["adj"]
    assert np.array_equal(adj.replay(c4["u0"], A), c4["replay_u0"])
    assert np.array_equal(adj.replay(c4["v"], A), c4["replay_v"])


def test_dot_product_against_the_oracle_operator(c4):
    lhs = float(c4["replay_v"] @ c4["w"])  # <L v, w>, L from the oracle (linear: Dirichlet 0)
    rhs = float(c4["v"] @ c4["LTw"])  # <v, L^T w>, L^T from the GPU's backward pass
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_gradient_against_oracle_finite_differences(c4):
    J, hu, ha = c4["J"], c4["hu"], c4["ha"]
    fd = c4["fd_jobs"]
    for k, d in enumerate(c4["dirs"]):
        q = (J(fd[2 * k]) - J(fd[2 * k + 1])) / (2 * hu)
        assert abs(q - float(c4["g0"] @ d)) <= 1e-6 * abs(q), (k, q, float(c4["g0"] @ d))
    base = 2 * len(c4["dirs"])
    for k in range(2):
        q = (J(fd[base + 2 * k]) - J(fd[base + 2 * k + 1])) / (2 * ha)
        assert abs(q - c4["ga"][k]) <= 1e-6 * abs(q), (k, q, c4["ga"][k])
