"""samurai's default mesh configuration (max_stencil_radius 2: mesh_config.hpp:388-393
raises the radius to 2 unless disable_minimal_ghost_width() is called) in the
oracle: the graduation gains the contiguous-boundary pass
(list_interval_to_refine_for_contiguous_boundary_cells, graduation.hpp:370-497)
and the ghost layers are two cells wide.  No golden output of the reference
covers this configuration, so the restatement is pinned by the properties the
reference's code states: after every adaptation, the second cell inward from a
leaf on the boundary lies in a leaf at least as fine as that leaf (the pass
refines coarser ones), the mesh stays 2:1 graded and tiles the box, and every
value stays finite.  With --refine-boundary the boundary stays at max_level
while the inside coarsens, which makes the pass refine a ring of cells: with
radius 1 the first property then fails on the same data, which shows the pass
at work."""
import numpy as np
import pytest

from advection_cases import ball_3d, shapes_2d
from oracle.pyoracle import OracleSim


def leaf_level_map(level, coords, maxl):
    dim = coords.shape[1]
    n = 1 << maxl
    grid = np.full((n,) * dim, -1, np.int16)
    for l in np.unique(level):
        s = 1 << (maxl - int(l))
        for c in coords[level == l]:
            sl = tuple(slice(int(c[d]) * s, (int(c[d]) + 1) * s) for d in reversed(range(dim)))
            grid[sl] = l
    return grid


def boundary_violations(level, coords, maxl):
    """leaves b of level L on the boundary whose cell b - 2 t (t the outward normal)
    lies in a coarser leaf"""
    dim = coords.shape[1]
    grid = leaf_level_map(level, coords, maxl)
    bad = 0
    for lv, c in zip(level, coords):
        n = 1 << int(lv)
        s = 1 << (maxl - int(lv))
        for d in range(dim):
            for t in (1, -1):
                if (t == 1 and c[d] != n - 1) or (t == -1 and c[d] != 0):
                    continue
                q = c.astype(np.int64).copy()
                q[d] -= 2 * t
                if q[d] < 0 or q[d] >= n:
                    continue
                fine = tuple(int(q[k]) * s for k in reversed(range(dim)))
                if grid[fine] < lv:
                    bad += 1
    return bad


def run(dim, radius, steps=4, refine_boundary=False):
    minl, maxl = (2, 7) if dim == 2 else (2, 5)
    o = OracleSim(dim, minl, maxl, radius, 1)
    o.set_refine_boundary(refine_boundary)
    lv, co, _ = o.cells()
    o.set_cell_values((shapes_2d(3, 10, 10) if dim == 2 else ball_3d(5))(lv, co))
    o.adapt(1e-3, 1.0)
    out = []
    a = [1.0, -0.5, 0.5][:dim]
    for _ in range(steps):
        lv, co, _ = o.cells()
        out.append((lv, co, o.cell_values()))
        o.update_ghost()
        o.upwind(a, 0.3 / (1 << maxl))
        o.adapt(1e-3, 1.0)
    return out, maxl


@pytest.mark.parametrize("dim,refine_boundary", [(2, False), (2, True), (3, False), (3, True)])
def test_contiguous_boundary_cells(dim, refine_boundary):
    states, maxl = run(dim, 2, refine_boundary=refine_boundary)
    for lv, co, v in states:
        assert boundary_violations(lv, co, maxl) == 0
        grid = leaf_level_map(lv, co, maxl)
        assert grid.min() >= 0 and np.all(np.isfinite(v))
        for ax in range(dim):
            assert np.abs(np.diff(grid.astype(np.int32), axis=ax)).max() <= 1
    if refine_boundary:
        states1, maxl = run(dim, 1, steps=1, refine_boundary=True)
        assert boundary_violations(states1[0][0], states1[0][1], maxl) > 0
