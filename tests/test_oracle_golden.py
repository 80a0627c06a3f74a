"""Pin the CPU oracle against the reference's committed golden outputs of
demos/FiniteVolume/advection_2d.cpp (min level 4, max level 10,
max_stencil_size 2, eps 2e-4, regularity 1, disc of radius 0.2 at (0.3,0.3),
a = (1,1), cfl 0.5, Tf = 0.01), for prediction radius 0 and 1.

The reference's own test compares these files with rel 1e-14, abs 1e-7
(tests/conftest.py:121-122).  Here the adapted meshes must be identical and
the fields must agree within that tolerance; the initial (adapted once)
fields are bit-identical.
"""
import os

import numpy as np
import pytest

from advection_cases import demo_time_loop, disc
from oracle.pyoracle import OracleSim

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _run(pred):
    s = OracleSim(2, 4, 10, max_stencil_radius=1, prediction_radius=pred)
    lv, co, _ = s.cells()
    s.set_cell_values(disc(lv, co))
    s.adapt(2e-4, 1.0)
    lv, co, _ = s.cells()
    init = (lv, co, s.cell_values())
    dt = 0.5 * (1.0 / (1 << 10))
    nt = demo_time_loop(s, dt, 0.01, 2e-4, 1.0, [1.0, 1.0])
    lv, co, _ = s.cells()
    return init, (lv, co, s.cell_values()), nt


@pytest.mark.parametrize("pred", [0, 1])
def test_oracle_matches_golden(pred):
    init, final, nt = _run(pred)
    assert nt == 21
    for (lv, co, u), name, exact in ((init, f"pred_{pred}_init", True), (final, f"pred_{pred}", False)):
        g = np.load(os.path.join(GOLD, name + ".npz"))
        assert len(lv) == len(g["u"]), name
        assert np.array_equal(lv, g["level"]), name
        assert np.array_equal(co[:, 0], g["i"]) and np.array_equal(co[:, 1], g["j"]), name
        assert not np.isnan(u).any()
        if exact:
            assert np.array_equal(u, g["u"]), name
        else:
            np.testing.assert_allclose(u, g["u"], rtol=1e-14, atol=1e-7)
            assert np.max(np.abs(u - g["u"])) <= 1e-15
