"""Output and restart files: samurai::save (io/hdf5.hpp) and samurai::dump /
load (io/restart.hpp), written and read by the library without libhdf5.

save is pinned to the reference's own golden files: after the advection_2d
demo (the golden replay), the file's /mesh/points and /mesh/connectivity are
byte-identical to the reference's (SHA-256 digests in the fixtures), u
matches within the reference test's tolerance, and the .xdmf text is
identical.  Files are decoded with the independent pure-Python reader of
tests/h5lite.py; the restart layout is compared with a restatement of
LevelCellArray (advection_cases.level_cell_array), and a run restarted from a
dump continues bit for bit."""
import hashlib
import os

import numpy as np
import pytest

from advection_cases import ball_3d, disc, level_cell_array, save_mesh_arrays, shapes_2d
from h5lite import H5

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import samurai_gb300

    samurai_gb300.lib()
    return samurai_gb300


def demo_run(sg, pred):
    """demos/FiniteVolume/advection_2d.cpp with --Tf 0.01 on the GPU"""
    g = sg.AdvectionSim(2, 4, 10, 1, pred)
    lv, co, _ = g.cells()
    g.set_cell_values(disc(lv, co))
    g.adapt(2e-4, 1.0)
    dt = 0.5 * (1.0 / (1 << 10))
    t, Tf = 0.0, 0.01
    while t != Tf:
        g.adapt(2e-4, 1.0)
        t += dt
        if t > Tf:
            dt += Tf - t
            t = Tf
        g.update_ghost()
        g.upwind([1.0, 1.0], dt, 0)
    return g


@pytest.mark.parametrize("pred", [0, 1])
def test_save_matches_golden_files(sg, tmp_path, pred):
    gold = np.load(os.path.join(GOLD, "pred_%d.npz" % pred))
    name = str(gold["file_name"])
    g = demo_run(sg, pred)
    sg.save(str(tmp_path), name, g.mesh, g.u)
    h = H5(os.path.join(str(tmp_path), name + ".h5"))
    assert h.keys("/mesh") == ["connectivity", "fields", "points"]
    pts = h.read("/mesh/points")
    conn = h.read("/mesh/connectivity")
    assert pts.dtype == np.dtype("<f8") and conn.dtype == np.dtype("<u8")
    assert len(pts) == int(gold["n_points"])
    assert hashlib.sha256(np.ascontiguousarray(pts).tobytes()).hexdigest() == str(gold["points_sha256"])
    assert hashlib.sha256(np.ascontiguousarray(conn).tobytes()).hexdigest() == str(gold["connectivity_sha256"])
    u = h.read("/mesh/fields/u")
    assert np.array_equal(u, g.cell_values())
    np.testing.assert_allclose(u, gold["u"], rtol=1e-14, atol=1e-7)
    xdmf = open(os.path.join(str(tmp_path), name + ".xdmf")).read()
    assert xdmf == str(gold["xdmf"])


@pytest.mark.parametrize("dim,minl,maxl", [(2, 2, 7), (3, 2, 5)])
def test_save_vector_and_scalar_fields(sg, tmp_path, dim, minl, maxl):
    """save(path, name, mesh, u, v): one dataset per component (<name>_<c>),
    points and connectivity as samurai numbers them (io/hdf5.hpp:85-144)."""
    mesh = sg.MRMesh(dim, minl, maxl, 1, 1)
    u = sg.make_scalar_field("u", mesh)
    v = sg.make_vector_field("v", mesh, 2)
    sg.make_bc(sg.Dirichlet(1), u, 0.0)
    sg.make_bc(sg.Dirichlet(1), v, 0.0, 0.0)
    lv, co, _ = mesh.cells()
    f = shapes_2d(3, 2, 2) if dim == 2 else ball_3d(4)
    u.set_cells(f(lv, co))
    v.set_cells(np.stack([0.5 * f(lv, co), -f(lv, co)], axis=1))
    sg.make_MRAdapt(u, v)(1e-3, 1.0)
    sg.save(str(tmp_path), "fields", mesh, u, v)
    h = H5(os.path.join(str(tmp_path), "fields.h5"))
    lv, co, _ = mesh.cells()
    rp, rc = save_mesh_arrays(lv, co, maxl)
    assert np.array_equal(h.read("/mesh/points"), rp)
    assert np.array_equal(h.read("/mesh/connectivity"), rc)
    assert sorted(h.keys("/mesh/fields")) == ["u", "v_0", "v_1"]
    vals = v.cell_values()
    assert np.array_equal(h.read("/mesh/fields/u"), u.cell_values())
    assert np.array_equal(h.read("/mesh/fields/v_0"), vals[:, 0])
    assert np.array_equal(h.read("/mesh/fields/v_1"), vals[:, 1])
    xdmf = open(os.path.join(str(tmp_path), "fields.xdmf")).read()
    assert ('TopologyType="%s"' % ("Quadrilateral" if dim == 2 else "Hexahedron")) in xdmf
    assert xdmf.count("<Attribute ") == 3


@pytest.mark.parametrize("dim,minl,maxl", [(2, 3, 8), (3, 2, 5)])
def test_dump_layout_and_restart(sg, tmp_path, dim, minl, maxl):
    """dump writes the leaf CellArray as LevelCellArray intervals and offsets
    and the fields' leaf values; load into a fresh mesh gives the same cells
    and values, and the restarted run continues bit for bit."""
    a = (1.0, 0.5) if dim == 2 else (1.0, 0.5, -0.25)
    dt = 0.4 / (1 << maxl)
    g = sg.AdvectionSim(dim, minl, maxl, 1, 1)
    w = sg.make_vector_field("w", g.mesh, 2)
    lv, co, _ = g.cells()
    f = shapes_2d(6, 2, 2) if dim == 2 else ball_3d(5)
    g.set_cell_values(f(lv, co))
    w.set_cells(np.stack([f(lv, co), 0.25 * f(lv, co)], axis=1))
    for _ in range(3):
        g.adaptation(1e-3, 1.0, w)
        g.update_ghost()
        g.upwind(a, dt)
    g.adaptation(1e-3, 1.0, w)
    sg.dump(str(tmp_path), "restart", g.mesh, g.u, w)

    # the file, decoded independently
    h = H5(os.path.join(str(tmp_path), "restart.h5"))
    assert int(h.read("/n_process")) == 1 and int(h.read("/mesh/dim")) == dim
    assert int(h.read("/mesh/min_level")) == minl and int(h.read("/mesh/max_level")) == maxl
    assert np.array_equal(h.read("/mesh/origin_point"), np.zeros(dim)) and float(h.read("/mesh/scaling_factor")) == 1.0
    for lev in range(maxl + 1):
        rows = g.mesh.intervals("cells", lev, with_index=True)
        if len(rows) == 0:
            assert not h.exists("/mesh/level/%d" % lev)
            continue
        ivs, offs = level_cell_array(rows, dim)
        for d in range(dim):
            data = h.read("/mesh/level/%d/dim/%d/intervals/data" % (lev, d))
            assert list(h.read("/mesh/level/%d/dim/%d/intervals/partition" % (lev, d))) == [0, len(data)]
            got = [(int(r["start"]), int(r["end"]), int(r["index"])) for r in data]
            assert got == ivs[d], "level %d dim %d intervals" % (lev, d)
            assert all(int(r["step"]) == 1 for r in data)
        for d in range(1, dim):
            assert list(h.read("/mesh/level/%d/dim/%d/offsets/data" % (lev, d))) == offs[d - 1]
    assert int(h.read("/fields/u/n_comp")) == 1 and int(h.read("/fields/w/n_comp")) == 2
    assert np.array_equal(h.read("/fields/u/data/data"), g.cell_values())
    assert np.array_equal(h.read("/fields/w/data/data"), w.cell_values().reshape(-1))

    # restart
    assert sg.restart_levels(str(tmp_path), "restart") == (dim, minl, maxl)
    r = sg.AdvectionSim(dim, minl, maxl, 1, 1)
    rw = sg.make_vector_field("w", r.mesh, 2)
    sg.load(str(tmp_path), "restart", r.mesh, r.u, rw)
    for x, y in zip(g.cells(), r.cells()):
        assert np.array_equal(x, y)
    assert np.array_equal(r.cell_values(), g.cell_values())
    assert np.array_equal(rw.cell_values(), w.cell_values())
    for step in range(3):
        for s, ww in ((g, w), (r, rw)):
            s.update_ghost()
            s.upwind(a, dt)
            s.adaptation(1e-3, 1.0, ww)
        for x, y in zip(g.cells(), r.cells()):
            assert np.array_equal(x, y), "step %d" % step
        assert np.array_equal(r.cell_values(), g.cell_values()), "step %d" % step
        assert np.array_equal(rw.cell_values(), w.cell_values()), "step %d" % step


def test_load_rejects_other_levels_and_missing_fields(sg, tmp_path):
    g = sg.AdvectionSim(2, 2, 6, 1, 1)
    g.set_cell_values(np.ones(g.nb_cells()))
    sg.dump(str(tmp_path), "r", g.mesh, g.u)
    other = sg.AdvectionSim(2, 2, 7, 1, 1)
    with pytest.raises(sg.SamuraiGpuError, match="levels"):
        sg.load(str(tmp_path), "r", other.mesh, other.u)
    same = sg.AdvectionSim(2, 2, 6, 1, 1)
    v = sg.make_scalar_field("v", same.mesh)
    with pytest.raises(sg.SamuraiGpuError, match="does not exist"):
        sg.load(str(tmp_path), "r", same.mesh, v)
    with pytest.raises(sg.SamuraiGpuError):
        sg.load(str(tmp_path), "missing", same.mesh, same.u)


def test_load_refuses_corrupted_restart_files(sg, tmp_path):
    """an interval outside the level's box, an offsets entry past the
    interval array and a truncated file are refused with an error; a valid
    file still loads afterwards"""
    g = sg.AdvectionSim(2, 2, 6, 1, 1)
    lv, co, _ = g.cells()
    g.set_cell_values(shapes_2d(9, 2, 2)(lv, co))
    g.adapt(1e-3, 1.0)
    sg.dump(str(tmp_path), "good", g.mesh, g.u)
    good = os.path.join(str(tmp_path), "good.h5")
    raw = open(good, "rb").read()
    h = H5(good)
    lev = max(l for l in range(7) if h.exists("/mesh/level/%d" % l))
    ivx = h.read("/mesh/level/%d/dim/0/intervals/data" % lev)
    offs = h.read("/mesh/level/%d/dim/1/offsets/data" % lev)
    at_iv = raw.find(ivx.tobytes())
    at_off = raw.find(offs.tobytes())
    assert at_iv > 0 and at_off > 0

    def corrupted(name, data):
        with open(os.path.join(str(tmp_path), name + ".h5"), "wb") as f:
            f.write(data)

    b = bytearray(raw)
    b[at_iv + 4:at_iv + 8] = np.int32(1 << 30).tobytes()  # end of the first x-interval
    corrupted("far", bytes(b))
    b = bytearray(raw)
    b[at_off + 8:at_off + 16] = np.uint64(1 << 40).tobytes()  # second offsets entry
    corrupted("offsets", bytes(b))
    corrupted("short", raw[: len(raw) // 2])
    for name, what in (("far", "outside"), ("offsets", "inconsistent"), ("short", None)):
        r = sg.AdvectionSim(2, 2, 6, 1, 1)
        with pytest.raises(sg.SamuraiGpuError, match=what):
            sg.load(str(tmp_path), name, r.mesh, r.u)
    r = sg.AdvectionSim(2, 2, 6, 1, 1)
    sg.load(str(tmp_path), "good", r.mesh, r.u)
    assert np.array_equal(r.cell_values(), g.cell_values())
