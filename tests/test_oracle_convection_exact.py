"""Known answer of the convection operators, on the oracle.

samurai's tests/test_fv_operators.cpp (check_convection_exact) states that the linear upwind convection with a
constant velocity v computes div(v u) = v . grad(u) exactly for a linear field u = sum_d b_d x_d: on the interior
cells of a uniform mesh of level 3 the result is the constant sum_d v_d b_d (b_d = d + 2, v_d = d + 1).  Here the
same is checked on the oracle's time step, u_new = u - dt * op(u) with dt = 1, for the flux form
(make_convection_upwind), the upwind operator form and, in 2D, the README's scheme: op(u) = u - u_new on the cells
whose neighbours are all inside the box.  The README's scheme (README.md:144-151) spells out backward differences
in x and y with unit velocity whatever a is, so its answer is sum_d b_d."""
import numpy as np
import pytest

from oracle.pyoracle import OracleSim


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_upwind_convection_of_a_linear_field_is_exact(dim, scheme):
    if scheme == 1 and dim != 2:
        pytest.skip("the README scheme is two-dimensional")
    level = 3
    n = 1 << level
    sim = OracleSim(dim, level - 1, level, 1, 1, dirichlet=0.0)
    grid = np.stack(np.meshgrid(*([np.arange(n)] * dim), indexing="ij"), axis=-1).reshape(-1, dim)[:, ::-1]
    sim.set_cells(np.full(len(grid), level, np.int32), grid.astype(np.int32))
    lv, co, _ = sim.cells()
    b = np.arange(dim) + 2.0
    v = np.arange(dim) + 1.0
    x = (co + 0.5) / n
    u0 = x @ b
    sim.set_cell_values(u0)
    sim.update_ghost()
    sim.upwind(v, 1.0, scheme)
    op = u0 - sim.cell_values()
    interior = np.all((co >= 1) & (co < n - 1), axis=1)
    assert interior.sum() > 0
    expected = float(b.sum()) if scheme == 1 else float(v @ b)
    np.testing.assert_allclose(op[interior], expected, rtol=0, atol=1e-10)
