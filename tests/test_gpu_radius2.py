"""samurai's default mesh configuration, max_stencil_radius 2 (mesh_config.hpp:
388-393: without disable_minimal_ghost_width() the radius is raised to 2): two
ghost layers (the second by polynomial extrapolation at the boundary, corner
blocks filled by the off-diagonal copies, bc/apply_field_bc.hpp:371-593) and the
contiguous-boundary graduation pass (graduation.hpp:370-497).  The GPU against
the oracle, bit for bit, on every mesh id, the leaf cells and values, through
adaptations and steps, in 2D and 3D, with and without --refine-boundary (which
makes the contiguous-boundary pass refine a ring of cells) and on a mesh with a
periodic axis."""
import numpy as np
import pytest

from advection_cases import ball_3d, shapes_2d
from gpu_util import compare_cells, compare_fields, compare_meshes
from oracle.pyoracle import OracleSim

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from samurai_gb300 import build

    build.build()
    import samurai_gb300

    return samurai_gb300


@pytest.mark.parametrize("dim,refine_boundary,periodic", [(2, False, None), (2, True, None), (3, False, None), (3, True, None),
                                                          (2, False, (True, False))])
def test_radius2_against_oracle(sg, dim, refine_boundary, periodic):
    minl, maxl = (2, 7) if dim == 2 else (2, 5)
    per = periodic or (False, False, False)
    g = sg.AdvectionSim(dim, minl, maxl, 2, 1, periodic=periodic)
    o = OracleSim(dim, minl, maxl, 2, 1, periodic=tuple(per) + (False,) * (3 - len(per)))
    g.mesh.set_refine_boundary(refine_boundary)
    o.set_refine_boundary(refine_boundary)
    compare_meshes(g, o, maxl, "uniform")
    lv, co, _ = o.cells()
    vals = (shapes_2d(3, 10, 10) if dim == 2 else ball_3d(5))(lv, co)
    g.set_cell_values(vals)
    o.set_cell_values(vals)
    a = [1.0, -0.5, 0.5][:dim]
    dt = 0.3 / (1 << maxl)
    assert g.adapt(1e-3, 1.0) == o.adapt(1e-3, 1.0)
    for it in range(4):
        compare_cells(g, o, "it %d" % it)
        g.update_ghost()
        o.update_ghost()
        compare_fields(g, o, "it %d ghosts" % it)
        g.upwind(a, dt)
        o.upwind(a, dt)
        compare_fields(g, o, "it %d upwind" % it, cells_only=True)
        assert g.adapt(1e-3, 1.0) == o.adapt(1e-3, 1.0), "it %d: Harten passes" % it
    compare_meshes(g, o, maxl, "final")
    compare_cells(g, o, "final")
    compare_fields(g, o, "final", cells_only=True)


def test_radius2_step_graph(sg):
    """the whole step as one graph on a radius-2 mesh gives the separate calls' results"""
    one, sep = sg.AdvectionSim(2, 2, 7, 2, 1), sg.AdvectionSim(2, 2, 7, 2, 1)
    lv, co, _ = one.cells()
    for s in (one, sep):
        s.mesh.set_refine_boundary(True)
        s.set_cell_values(shapes_2d(5, 8, 8)(lv, co))
    dt = 0.3 / (1 << 7)
    for it in range(5):
        assert one.step(1e-3, 1.0, [1.0, 0.5], dt) == sep.adapt(1e-3, 1.0)
        sep.update_ghost()
        sep.upwind([1.0, 0.5], dt)
        assert np.array_equal(one.cell_values(), sep.cell_values()), "step %d" % it


def test_radius2_adjoint_is_refused(sg):
    s = sg.AdvectionSim(2, 2, 6, 2, 1)
    with pytest.raises(sg.SamuraiGpuError, match="ghost width of 1"):
        sg.Adjoint(s.u)
