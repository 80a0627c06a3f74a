"""Known answers of the Dirichlet boundary ghosts, on the oracle.

samurai's tests/test_bc_ghost_values.cpp checks that the ghosts next to the boundary hold the exact values of a
function the boundary condition reproduces: Dirichlet<1> (ghost = 2 v - u) is exact on a function linear in the
normal coordinate, and the further ghost layers of a wider stencil, filled by polynomial extrapolation
(bc/apply_field_bc.hpp:531-593), are exact on it too; the checks cover a uniform mesh and an adapted one whose
boundary crosses levels, and look at the ghosts beside the boundary leaves of every level.  The oracle restates
the same operations; here its ghost update is checked the same way with u = 1 + 3 x and the constant Dirichlet
value v = u(x = 0) = 1, on the -x side of the box (the value of the other sides differs), ghost widths 1 and 2."""
import numpy as np
import pytest

from oracle.pyoracle import OracleSim


def f(level, coords):
    x = (coords[:, 0] + 0.5) / (1 << level)
    return 1.0 + 3.0 * x


def storage_index(sim, maxl):
    """{(level, coords...): index} of every reference cell in samurai's storage order (level, rows, x)"""
    dim = sim.dim
    out, k = {}, 0
    for l in range(maxl + 1):
        for row in sim.intervals("reference", l):
            rest = tuple(int(v) for v in row[2:2 + dim - 1])
            for x in range(int(row[0]), int(row[1])):
                out[(l, x) + rest] = k
                k += 1
    return out


def make_problem(dim, radius, adapted):
    minl, maxl = (2, 5) if adapted else (3, 4)
    sim = OracleSim(dim, minl, maxl, radius, 1, dirichlet=1.0)
    if adapted:
        # the mesh of the indicator of the ball |x| < 0.3 (Dirichlet 0) adapted with eps 1e-4, as in samurai's
        # test: its boundary leaves span several levels
        phi = OracleSim(dim, minl, maxl, radius, 1, dirichlet=0.0)
        lv, co, _ = phi.cells()
        c = (co + 0.5) / (1 << lv)[:, None]
        phi.set_cell_values((np.sqrt((c * c).sum(axis=1)) < 0.3).astype(np.float64))
        phi.adapt(1e-4, 1.0)
        lv, co, _ = phi.cells()
        sim.set_cells(lv, co)
    else:
        n = 1 << maxl
        grid = np.stack(np.meshgrid(*([np.arange(n)] * dim), indexing="ij"), axis=-1).reshape(-1, dim)[:, ::-1]
        sim.set_cells(np.full(len(grid), maxl, np.int32), grid.astype(np.int32))
    return sim, maxl


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("radius", [1, 2])
@pytest.mark.parametrize("adapted", [False, True])
def test_dirichlet_ghosts_are_exact_on_linear_functions(dim, radius, adapted):
    sim, maxl = make_problem(dim, radius, adapted)
    lv, co, _ = sim.cells()
    if adapted:
        assert len(np.unique(lv[co[:, 0] == 0])) > 1, "the -x boundary should cross levels"
    sim.set_cell_values(f(lv, co))
    sim.update_ghost()
    u = sim.field()
    index = storage_index(sim, maxl)
    checked = 0
    for l in np.unique(lv):
        bnd = co[(lv == l) & (co[:, 0] == 0)]  # leaves of level l on the -x boundary
        for layer in range(1, radius + 1):
            g = bnd.copy()
            g[:, 0] = -layer
            keys = [(int(l),) + tuple(int(v) for v in c) for c in g]
            idx = [index[k] for k in keys if k in index]
            assert len(idx) == len(keys), "every ghost of the layer is a reference cell"
            want = f(int(l), g)
            np.testing.assert_allclose(u[idx], want, rtol=0, atol=1e-11)
            checked += len(idx)
    assert checked > 0
