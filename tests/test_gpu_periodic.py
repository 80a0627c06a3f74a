"""Periodic axes on the GPU (mesh_config<dim>().periodic(...)), bit for bit
against the oracle: every MRMesh id of the uniform and of the adapted meshes,
the ghost values after update_ghost_mr (periodic copies, boundary conditions
on the other axes only), details and tags of a Harten pass, and a few time
steps.  The oracle's periodic restatement is itself checked by translation
covariance (tests/test_oracle_periodic.py)."""
import numpy as np
import pytest

from gpu_util import compare_cells, compare_fields, compare_meshes
from oracle.pyoracle import OracleSim

pytestmark = pytest.mark.gpu

CASES = [
    (2, 2, 7, (True, True, False)),
    (2, 3, 8, (True, False, False)),
    (2, 2, 7, (False, True, False)),
    (3, 2, 5, (True, True, True)),
    (3, 2, 5, (False, True, False)),
    (3, 3, 6, (True, False, True)),
]


@pytest.fixture(scope="module")
def sg():
    import samurai_gb300

    samurai_gb300.lib()
    return samurai_gb300


def pair(sg, dim, minl, maxl, per, dirichlet=0.0):
    g = sg.AdvectionSim(dim, minl, maxl, 1, 1, 1, dirichlet, periodic=per[:dim])
    o = OracleSim(dim, minl, maxl, 1, 1, 1, dirichlet, periodic=per)
    return g, o


def near_boundary(lv, co, dim):
    """a bump and a plateau that straddle the x = 0 / x = 1 and y = 0 sides"""
    c = (co + 0.5) / (1 << lv)[:, None]
    r2 = 0.0
    for d in range(dim):
        x = c[:, d]
        r2 = r2 + np.minimum(abs(x - 0.05), 1 - abs(x - 0.05)) ** 2
    return np.exp(-r2 / 0.004) + 0.5 * (r2 < 0.01)


@pytest.mark.parametrize("dim,minl,maxl,per", CASES)
def test_periodic_uniform_mesh_ids(sg, dim, minl, maxl, per):
    g, o = pair(sg, dim, minl, maxl, per)
    compare_meshes(g, o, maxl, "uniform periodic")


@pytest.mark.parametrize("dim,minl,maxl,per", CASES)
def test_periodic_adaptation_and_steps(sg, dim, minl, maxl, per):
    g, o = pair(sg, dim, minl, maxl, per, dirichlet=0.25)
    lv, co, _ = o.cells()
    vals = near_boundary(lv, co, dim)
    o.set_cell_values(vals)
    g.set_cell_values(vals)
    a = (-1.0, 0.5) if dim == 2 else (-1.0, 0.5, 0.75)
    dt = 0.4 / (1 << maxl)
    for step in range(4):
        assert g.adapt(1e-3, 1.0) == o.adapt(1e-3, 1.0), "step %d: Harten passes" % step
        compare_meshes(g, o, maxl, "step %d" % step)
        compare_cells(g, o, "step %d" % step)
        compare_fields(g, o, "step %d leaves" % step, cells_only=True)
        g.update_ghost()
        o.update_ghost()
        compare_fields(g, o, "step %d ghosts" % step)
        g.upwind(a, dt)
        o.upwind(a, dt)
        compare_fields(g, o, "step %d upwind" % step, cells_only=True)


@pytest.mark.parametrize("dim,minl,maxl,per", CASES[:4])
def test_periodic_detail_and_tags(sg, dim, minl, maxl, per):
    """details on every reference cell and tags (after the periodic tag
    exchange and the maximum operator) of a converged Harten pass"""
    g, o = pair(sg, dim, minl, maxl, per)
    lv, co, _ = o.cells()
    vals = near_boundary(lv, co, dim)
    o.set_cell_values(vals)
    g.set_cell_values(vals)
    o.adapt(1e-3, 1.0)
    g.adapt(1e-3, 1.0)
    for ite in range(5):
        ro = o.harten(ite, 1e-3, 1.0)
        assert g.harten(ite, 1e-3, 1.0) == ro
        if ro:
            do, dg = o.detail(), g.detail()
            ok = ~np.isnan(do)
            assert np.array_equal(dg[ok], do[ok])
            assert np.array_equal(o.tag(), g.tag())
            break
    else:
        pytest.fail("no converged Harten pass")
    compare_cells(g, o, "after harten")


def test_periodic_mesh_rejects_flux_form_and_adjoint(sg):
    g = sg.AdvectionSim(2, 2, 6, 1, 1, 1, 0.0, periodic=(True, True))
    g.set_cell_values(np.ones(g.nb_cells()))
    g.update_ghost()
    with pytest.raises(sg.SamuraiGpuError, match="periodic"):
        g.upwind((1.0, 1.0), 0.01, sg.CONVECTION)
    with pytest.raises(sg.SamuraiGpuError, match="periodic"):
        sg.Adjoint(g.u, 8)
