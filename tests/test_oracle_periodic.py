"""Periodic meshes in the oracle (mesh_config::periodic): the restatement of
the periodic parts of mesh construction (mr/mesh.hpp:276-368), ghost update
(algorithm/update_periodic.hpp, update_ghost_mr.hpp:195-237), tag
finalisation and graduation (graduation.hpp:309-318) is checked by
translation covariance: translating the initial field along the periodic
axes by a multiple of the cell size of level min_level - 2 (the coarsest
level of the reference mesh) translates the adapted meshes and every leaf
value of the run, bit for bit.  Dirichlet axes are not translated."""
import numpy as np
import pytest

from oracle.pyoracle import OracleSim


def run(dim, minl, maxl, per, shift, steps=3):
    o = OracleSim(dim, minl, maxl, 1, 1, 1, 0.0, periodic=per)
    lv, co, _ = o.cells()
    n = 1 << maxl
    c = (co + 0.5) / (1 << lv)[:, None]
    r2 = 0.0
    for d in range(dim):
        x = (c[:, d] - shift[d] / n) % 1.0
        r2 = r2 + np.minimum(abs(x - 0.1), 1 - abs(x - 0.1)) ** 2
    o.set_cell_values(np.exp(-r2 / 0.004) + (r2 < 0.01))
    a = (-1.0, 0.5) if dim == 2 else (-1.0, 0.5, 0.25)
    o.adapt(1e-3, 1.0)
    for _ in range(steps):
        o.update_ghost()
        o.upwind(a, 0.4 / n)
        o.adapt(1e-3, 1.0)
    lv, co, _ = o.cells()
    return lv, co, o.cell_values()


def canonical(lv, co, u, shift, maxl):
    cb = co.copy()
    for d in range(co.shape[1]):
        cb[:, d] = (co[:, d] - (shift[d] >> (maxl - lv))) % (1 << lv)
    k = np.lexsort(tuple(cb[:, d] for d in range(co.shape[1])) + (lv,))
    return lv[k], cb[k], u[k]


@pytest.mark.parametrize("dim,minl,maxl,per", [(2, 2, 7, (True, True, False)), (2, 3, 7, (True, False, False)),
                                               (2, 3, 7, (False, True, False)), (3, 2, 5, (True, True, True)),
                                               (3, 2, 5, (False, True, False))])
def test_periodic_translation_covariance(dim, minl, maxl, per):
    shift = [3 * (1 << (maxl - minl + 2)) if (d < dim and per[d]) else 0 for d in range(3)]
    base = canonical(*run(dim, minl, maxl, per, (0, 0, 0)), (0, 0, 0), maxl)
    moved = canonical(*run(dim, minl, maxl, per, shift), shift, maxl)
    assert np.array_equal(base[0], moved[0]) and np.array_equal(base[1], moved[1])
    assert np.array_equal(base[2], moved[2])


def test_periodic_mesh_wraps_the_reference():
    """Fine cells next to the x = 1 side put periodic ghosts of their level on
    the x = 0 side (mr/mesh.hpp:294-317): there the reference mesh of a
    periodic axis holds cells of the finest level, a Dirichlet one does not."""
    def finest_reference_near_zero(per):
        o = OracleSim(2, 2, 6, 1, 1, 1, 0.0, periodic=per)
        lv, co, _ = o.cells()
        c = (co + 0.5) / (1 << lv)[:, None]
        o.set_cell_values(np.exp(-((c[:, 0] - 0.99) ** 2 + (c[:, 1] - 0.5) ** 2) / 0.001))
        o.adapt(1e-3, 1.0)
        iv = o.intervals("reference", 6)
        return bool(np.any((iv[:, 0] <= 0) & (iv[:, 1] > 0)))

    assert finest_reference_near_zero((True, False, False))
    assert not finest_reference_near_zero((False, False, False))
