"""The oracle's restatement of make_convection_upwind (flux form with
level-jump interfaces), checked on the CPU against the properties the
reference's own tests state for it: a constant field with a matching
Dirichlet value is a steady state everywhere, level jumps included
(test_fv_operators.cpp:1013-1052); the flux form is conservative (the
volume-weighted sum of the operator is the boundary flux, zero for a field
that vanishes at the boundary); and on a uniform mesh it is the same upwind
difference as the operator form upwind(a, u)."""
import numpy as np
import pytest

from advection_cases import cell_volumes, disc
from oracle.pyoracle import OracleSim


def adapted(dim, minl, maxl, dirichlet=0.0, xc=0.5, eps=1e-3):
    o = OracleSim(dim, minl, maxl, 1, 1, 1, dirichlet)
    lv, co, _ = o.cells()
    c = (co + 0.5) / (1 << lv)[:, None]
    r2 = ((c - xc) ** 2).sum(axis=1)
    o.set_cell_values(np.where(r2 <= 0.2 ** 2, 1.0, 0.0) + np.exp(-r2 / 0.01))
    o.adapt(eps, 1.0)
    return o


def operator_values(o, a):
    """conv(u) on the leaf cells: unp1 = u - dt conv(u) with dt = 1"""
    o.update_ghost()
    u = o.cell_values()
    o.upwind(a, 1.0, 2)
    return u - o.cell_values()


@pytest.mark.parametrize("dim,a", [(2, (1.0, 2.0)), (2, (-0.75, 0.5)), (3, (1.0, -0.5, 0.25))])
def test_constant_field_is_steady(dim, a):
    c = 2.5
    o = adapted(dim, 2, 6 if dim == 2 else 5, dirichlet=c, eps=1e-3 if dim == 2 else 2e-2)
    lv, _, _ = o.cells()
    assert len(np.unique(lv)) > 1, "the mesh must have level jumps"
    o.set_cell_values(np.full(o.nb_cells(), c))
    out = operator_values(o, a)
    assert np.max(np.abs(out)) <= 1e-12 * c * (1 << int(lv.max()))


@pytest.mark.parametrize("dim,a", [(2, (1.0, 0.7)), (2, (-1.0, 0.3)), (3, (0.5, -1.0, 0.8))])
def test_flux_form_is_conservative(dim, a):
    o = adapted(dim, 2, 7 if dim == 2 else 5, eps=1e-3 if dim == 2 else 2e-2)
    lv, _, _ = o.cells()
    assert len(np.unique(lv)) > 1
    out = operator_values(o, a)
    vol = cell_volumes(lv, dim)
    total = float(np.sum(vol * out))
    scale = float(np.sum(vol * np.abs(out)))
    assert scale > 0
    # the field is ~exp(-0.2/0.01) at the boundary: boundary fluxes are negligible
    assert abs(total) <= 1e-9 * scale


@pytest.mark.parametrize("a", [(1.0, 0.5), (-0.5, -1.0)])
def test_uniform_mesh_matches_operator_form(a):
    o1 = OracleSim(2, 5, 5, 1, 1)
    o2 = OracleSim(2, 5, 5, 1, 1)
    lv, co, _ = o1.cells()
    vals = disc(lv, co, 0.5, 0.5, 0.25)
    for o in (o1, o2):
        o.set_cell_values(vals)
        o.update_ghost()
    o1.upwind(a, 1e-3, 0)
    o2.upwind(a, 1e-3, 2)
    np.testing.assert_allclose(o2.cell_values(), o1.cell_values(), rtol=1e-13, atol=1e-15)
