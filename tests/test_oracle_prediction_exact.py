"""Known answers of the ghost update's projection and prediction, on the oracle.

samurai's own round-trip test (tests/test_projection_prediction_roundtrip.cpp) states the accuracy of the two
operators: the projection reproduces cell averages of any polynomial exactly, and the prediction of stencil
radius s reproduces cell averages of polynomials of per-axis degree <= 2s.  Here the same facts are checked on
the oracle's update_ghost_mr: a mesh of one level with a block of the next finer level inside it, leaf values
set to exact cell averages of u = prod_d (1 + 2 x_d + 3 x_d^2) (per-axis degree 2), the block far from the
boundary.  After the ghost update, every projected cell of the coarse level and every predicted ghost of the
fine level (the reference cells inside the box that are neither leaves nor projected cells) must hold the exact
cell average of u, up to rounding; with prediction radius 0 the same holds for a constant."""
import numpy as np
import pytest

from oracle.pyoracle import OracleSim


def antideriv(t):
    # A'(t) = 1 + 2 t + 3 t^2
    return t + t * t + t * t * t


def cell_average(level, coords, degree2=True):
    h = 1.0 / (1 << level)
    out = np.ones(coords.shape[0])
    if not degree2:
        return out * 3.25
    for d in range(coords.shape[1]):
        a = coords[:, d] * h
        out *= (antideriv(a + h) - antideriv(a)) / h
    return out


def storage_cells(sim, maxl):
    """(level, coords) of every reference cell in samurai's storage order: level by level, rows, then x"""
    dim = sim.dim
    levels, coords = [], []
    for l in range(maxl + 1):
        for row in sim.intervals("reference", l):
            x0, x1 = int(row[0]), int(row[1])
            n = x1 - x0
            c = np.zeros((n, dim), np.int64)
            c[:, 0] = np.arange(x0, x1)
            for d in range(1, dim):
                c[:, d] = row[1 + d]
            levels.append(np.full(n, l))
            coords.append(c)
    return np.concatenate(levels), np.concatenate(coords)


def member(sim, mesh_id, level, coords):
    """whether each cell of `coords` (at `level`) belongs to mesh id `mesh_id`"""
    dim = coords.shape[1]
    keys = set()
    for row in sim.intervals(mesh_id, level):
        for x in range(int(row[0]), int(row[1])):
            keys.add((x,) + tuple(int(v) for v in row[2:2 + dim - 1]))
    return np.array([tuple(int(v) for v in c) in keys for c in coords], dtype=bool)


def block_mesh(dim, coarse, lo, hi):
    """leaves: the uniform mesh of level `coarse` with the block [lo, hi)^dim of its cells refined once"""
    n = 1 << coarse
    grid = np.stack(np.meshgrid(*([np.arange(n)] * dim), indexing="ij"), axis=-1).reshape(-1, dim)[:, ::-1]
    inside = np.all((grid >= lo) & (grid < hi), axis=1)
    keep = grid[~inside]
    fine = []
    for c in grid[inside]:
        for k in range(1 << dim):
            fine.append([2 * c[d] + ((k >> d) & 1) for d in range(dim)])
    fine = np.array(fine)
    level = np.concatenate([np.full(len(keep), coarse), np.full(len(fine), coarse + 1)]).astype(np.int32)
    coords = np.concatenate([keep, fine]).astype(np.int32)
    return level, coords


@pytest.mark.parametrize("dim,coarse,lo,hi", [(2, 5, 8, 24), (3, 3, 2, 6)])
@pytest.mark.parametrize("pred", [1, 0])
def test_projection_and_prediction_are_exact(dim, coarse, lo, hi, pred):
    fine = coarse + 1
    sim = OracleSim(dim, coarse - 1, fine, 1, pred)
    level, coords = block_mesh(dim, coarse, lo, hi)
    sim.set_cells(level, coords)
    lv, co, _ = sim.cells()
    sim.set_cell_values(cell_average(lv, co, degree2=(pred == 1)))
    sim.update_ghost()
    u = sim.field()
    slev, scoord = storage_cells(sim, fine)
    assert len(u) == len(slev)
    checked = 0
    for l, mesh_id in ((coarse, "proj_cells"), (fine, "reference")):
        sel = slev == l
        c = scoord[sel]
        n = 1 << l
        inbox = np.all((c >= 0) & (c < n), axis=1)
        if mesh_id == "reference":
            # predicted ghosts: inside the box, neither leaves nor projected cells
            mask = inbox & ~member(sim, "cells", l, c) & ~member(sim, "proj_cells", l, c)
        else:
            mask = inbox & member(sim, "proj_cells", l, c)
        assert mask.sum() > 0, (l, mesh_id)
        got = u[sel][mask]
        want = cell_average(np.full(mask.sum(), l), c[mask], degree2=(pred == 1))
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-13)
        checked += int(mask.sum())
    assert checked > 0
