"""--refine-boundary in the oracle (keep_boundary_refined, mr/adapt.hpp:245-274,
341-346): the leaves of max_level within max_stencil_radius cells of the domain
boundary are tagged keep in every Harten pass, so an adaptation that starts
from the uniform max_level mesh leaves the whole boundary layer at max_level,
while without the flag the same data coarsens it."""
import numpy as np
import pytest

from advection_cases import ball_3d, readme_square
from oracle.pyoracle import OracleSim


def boundary_layer_levels(o, maxl, r):
    """levels of the leaves that meet the layer of width r cells (at max_level) along the boundary"""
    lv, co, _ = o.cells()
    n = 1 << maxl
    s = np.left_shift(1, maxl - lv.astype(np.int64))[:, None]
    lo = co.astype(np.int64) * s  # finest-level extent [lo, lo + s) of each leaf
    hi = lo + s
    near = np.any((lo < r) | (hi > n - r), axis=1)
    return lv[near]


@pytest.mark.parametrize("dim", [2, 3])
def test_boundary_layer_stays_at_max_level(dim):
    minl, maxl = (2, 6) if dim == 2 else (2, 5)
    f = readme_square if dim == 2 else ball_3d(3)
    levels = {}
    for rb in (False, True):
        o = OracleSim(dim, minl, maxl)
        o.set_refine_boundary(rb)
        lv, co, _ = o.cells()
        o.set_cell_values(f(lv, co))
        o.adapt(1e-3, 1.0)
        levels[rb] = boundary_layer_levels(o, maxl, 1)
    assert np.all(levels[True] == maxl)
    assert np.any(levels[False] < maxl)
