"""The launch-shape autotuner (sg_autotune): it keeps the fastest of the shapes it
times, leaves the problem in the state it found, and a launch shape changes no
result (every shape gives the same meshes and values, bit for bit); a later mesh
of the same device and levels starts from the cached choice."""
import numpy as np
import pytest

from advection_cases import shapes_2d

pytestmark = pytest.mark.gpu

EPS, REG, A = 1e-4, 2.0, (1.0, 0.5)


@pytest.fixture(scope="module")
def sg():
    from samurai_gb300 import build

    build.build()
    import samurai_gb300

    return samurai_gb300


def problem(sg, maxl=9):
    s = sg.AdvectionSim(2, 3, maxl)
    lv, co, _ = s.cells()
    s.set_cell_values(shapes_2d(61, 8, 8)(lv, co))
    s.adapt(EPS, REG)
    return s


def test_autotune_keeps_state_and_results(sg):
    dt = 0.5 / (1 << 9)
    tuned, plain = problem(sg), problem(sg)
    for s in (tuned, plain):
        for _ in range(3):
            s.step(EPS, REG, A, dt)
    before = tuned.cells(), tuned.cell_values()
    d_ms, t_ms, shape = tuned.autotune(EPS, REG, A, dt, steps=4)
    assert 0 < t_ms <= d_ms
    assert shape["block"] in (128, 256, 512) and shape["max_blocks"] > 0
    after = tuned.cells(), tuned.cell_values()
    for x, y in zip(before[0], after[0]):
        assert np.array_equal(x, y)
    assert np.array_equal(before[1], after[1])
    # any launch shape gives the same results
    plain.mesh.launch_shape()
    for it in range(6):
        assert tuned.step(EPS, REG, A, dt) == plain.step(EPS, REG, A, dt)
        lt, ct, it_ = tuned.cells()
        lp, cp, ip = plain.cells()
        assert np.array_equal(lt, lp) and np.array_equal(ct, cp) and np.array_equal(it_, ip), "step %d: cells" % it
        assert np.array_equal(tuned.cell_values(), plain.cell_values()), "step %d: values" % it
    # a new mesh of the same device and levels starts from the cached shape
    assert problem(sg).mesh.launch_shape() == tuned.mesh.launch_shape()


@pytest.mark.parametrize("block,fuse,pairs", [(128, 512, 1), (512, 32, 0), (256, 0, 0)])
def test_launch_shapes_give_identical_results(sg, monkeypatch, block, fuse, pairs):
    """shapes set through the environment (an override of the cache) change no
    bit, including one-level tag finalisation launches instead of pairs"""
    monkeypatch.setenv("SG_BLOCK", str(block))
    monkeypatch.setenv("SG_FUSE_WORDS_FIELD", str(fuse))
    monkeypatch.setenv("SG_FUSE_WORDS_MAX", str(fuse))
    monkeypatch.setenv("SG_MAX_BLOCKS", "300")
    monkeypatch.setenv("SG_LEVEL_PAIRS", str(pairs))
    a = problem(sg, 8)
    for k in ("SG_BLOCK", "SG_FUSE_WORDS_FIELD", "SG_FUSE_WORDS_MAX", "SG_MAX_BLOCKS", "SG_LEVEL_PAIRS"):
        monkeypatch.delenv(k)
    b = problem(sg, 8)
    assert a.mesh.launch_shape()["block"] == block
    assert a.mesh.launch_shape()["level_pairs"] == bool(pairs)
    dt = 0.5 / (1 << 8)
    for it in range(5):
        assert a.step(EPS, REG, A, dt) == b.step(EPS, REG, A, dt)
        assert np.array_equal(a.cell_values(), b.cell_values()), "step %d" % it
