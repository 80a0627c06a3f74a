"""samurai's named timers (timers.hpp:111-1036; the scopes of mr/adapt.hpp:151-387,
update_ghost_mr.hpp:263 and the field expression) and the per-launch kernel
trace: the per-phase GPU times must account for the step, phase by phase."""
import time

import pytest

from advection_cases import shapes_2d

pytestmark = pytest.mark.gpu

NESTED = ["ghost update", "detail computation", "tag cells", "tag finalization", "mesh update", "make_graduation", "mesh construction",
          "fields update"]


@pytest.fixture(scope="module")
def sim():
    import samurai_gb300 as sg

    s = sg.AdvectionSim(2, 3, 9)
    lv, co, _ = s.cells()
    s.set_cell_values(shapes_2d(41, 6, 6)(lv, co))
    s.adapt(1e-4, 2.0)
    return s


def step(s):
    s.adapt(1e-4, 2.0)
    s.update_ghost()
    s.upwind([1.0, 0.5], 0.5 / (1 << 9))


def test_timers_add_up_to_the_step(sim):
    for _ in range(3):
        step(sim)
    sim.mesh.synchronize()
    sim.mesh.timers(enable=True, reset=True)
    n = 6
    t0 = time.perf_counter()
    for _ in range(n):
        step(sim)
    sim.mesh.synchronize()
    wall_ms = 1e3 * (time.perf_counter() - t0)
    t = sim.mesh.timers(enable=False)
    assert t["mesh adaptation"][1] == n and t["field expressions"][1] == n
    for name in ["mesh adaptation", "field expressions", "ghost update", "detail computation", "tag cells", "mesh update"]:
        assert t[name][0] > 0.0, name
    adapt_ms = t["mesh adaptation"][0]
    nested_ms = sum(t[k][0] for k in NESTED)
    # the phases are disjoint parts of the adaptation (each bracketed by events on the mesh stream)
    assert nested_ms <= 1.02 * adapt_ms + 0.05, (nested_ms, adapt_ms)
    # ... and cover most of it: what is left is host work between launches, not hidden kernels
    assert nested_ms >= 0.5 * adapt_ms, (nested_ms, adapt_ms)
    # the device-timed phases fit in the wall-clock time of the steps
    assert adapt_ms + t["field expressions"][0] <= 1.02 * wall_ms + 0.05, (adapt_ms, wall_ms)


def test_kernel_trace_accounts_for_the_step(sim):
    step(sim)
    sim.mesh.kernel_trace(True)  # the traced launch sequences are captured on first use
    step(sim)
    sim.mesh.kernel_trace(False)
    sim.mesh.synchronize()
    sim.mesh.kernel_trace(True)
    t0 = time.perf_counter()
    step(sim)
    sim.mesh.synchronize()
    wall_ms = 1e3 * (time.perf_counter() - t0)
    rows, valid = sim.mesh.kernel_trace(False)
    assert valid
    names = {r[0] for r in rows}
    for k in ("ghost_level", "predict", "detail", "criteria", "upwind", "update_fields", "scan_write"):
        assert k in names, k
    launches = sum(r[1] for r in rows)
    assert launches > 20
    total = sum(r[2] for r in rows)
    assert 0.0 < total <= 1.02 * wall_ms + 0.05, (total, wall_ms)
    assert all(r[2] >= 0.0 for r in rows)
