"""The samurai demo program (demos/FiniteVolume/advection_2d.cpp) written
against the C++ drop-in header include/samurai_gb300/samurai.hpp: it must
compile unchanged in its samurai calls (CPU test) and reproduce the
reference's golden meshes on the GPU."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "advection_2d.cpp")
VSRC = os.path.join(ROOT, "tests", "cpp", "vector_advection_2d.cpp")
ISRC = os.path.join(ROOT, "tests", "cpp", "intervals_2d.cpp")
FSRC = os.path.join(ROOT, "tests", "cpp", "fields_api_2d.cpp")
GOLD = os.path.join(ROOT, "tests", "golden")


def compile_demo(tmp_path, src=SRC):
    from samurai_gb300 import build

    lib = build.build()
    exe = os.path.join(str(tmp_path), os.path.splitext(os.path.basename(src))[0])
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"), src, "-L" + os.path.dirname(lib), "-lsamurai_gpu",
           "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    subprocess.check_call(cmd)
    return exe


def test_demo_compiles(tmp_path):
    exe = compile_demo(tmp_path)
    assert os.path.exists(exe)


def test_vector_demo_compiles(tmp_path):
    exe = compile_demo(tmp_path, VSRC)
    assert os.path.exists(exe)


def test_interval_program_compiles(tmp_path):
    exe = compile_demo(tmp_path, ISRC)
    assert os.path.exists(exe)


def test_fields_api_program_compiles(tmp_path):
    exe = compile_demo(tmp_path, FSRC)
    assert os.path.exists(exe)


@pytest.mark.gpu
@pytest.mark.parametrize("pred", [0, 1])
def test_demo_matches_golden(tmp_path, pred):
    exe = compile_demo(tmp_path)
    out = os.path.join(str(tmp_path), "out.txt")
    subprocess.check_call([exe, str(pred), out])
    lines = open(out).read().split("\n")
    assert int(lines[0]) == 21
    rows = np.array([[float(v) for v in l.split()] for l in lines[1:] if l.strip()])
    g = np.load(os.path.join(GOLD, "pred_%d.npz" % pred))
    assert np.array_equal(rows[:, 0].astype(int), g["level"])
    assert np.array_equal(rows[:, 1].astype(int), g["i"]) and np.array_equal(rows[:, 2].astype(int), g["j"])
    np.testing.assert_allclose(rows[:, 3], g["u"], rtol=1e-14, atol=1e-7)


@pytest.mark.gpu
def test_demo_save_matches_golden_files(tmp_path):
    """The demo's samurai::save through the C++ header: the .h5 mesh datasets
    are byte-identical to the reference's golden file (SHA-256 digests), u is
    within the reference test's tolerance and the .xdmf text is identical; the
    demo's dump / load round trip reproduces its cells and values."""
    import hashlib
    import sys

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from h5lite import H5

    exe = compile_demo(tmp_path)
    out = os.path.join(str(tmp_path), "out.txt")
    g = np.load(os.path.join(GOLD, "pred_0.npz"))
    name = str(g["file_name"])
    subprocess.check_call([exe, "0", out, "upwind", str(tmp_path), name])
    h = H5(os.path.join(str(tmp_path), name + ".h5"))
    pts, conn = h.read("/mesh/points"), h.read("/mesh/connectivity")
    assert hashlib.sha256(np.ascontiguousarray(pts).tobytes()).hexdigest() == str(g["points_sha256"])
    assert hashlib.sha256(np.ascontiguousarray(conn).tobytes()).hexdigest() == str(g["connectivity_sha256"])
    np.testing.assert_allclose(h.read("/mesh/fields/u"), g["u"], rtol=1e-14, atol=1e-7)
    assert open(os.path.join(str(tmp_path), name + ".xdmf")).read() == str(g["xdmf"])


@pytest.mark.gpu
def test_demo_flux_form_matches_oracle(tmp_path):
    """The demo with unp1 = u - dt * conv(u), conv = make_convection_upwind,
    against the oracle running the same loop: identical cells and values."""
    from advection_cases import demo_time_loop, disc
    from oracle.pyoracle import OracleSim

    exe = compile_demo(tmp_path)
    out = os.path.join(str(tmp_path), "out.txt")
    subprocess.check_call([exe, "1", out, "convection"])
    lines = open(out).read().split("\n")
    rows = np.array([[float(v) for v in l.split()] for l in lines[1:] if l.strip()])
    o = OracleSim(2, 4, 10, 1, 1)
    lv, co, _ = o.cells()
    o.set_cell_values(disc(lv, co))
    o.adapt(2e-4, 1.0)
    nt = demo_time_loop(o, 0.5 / 1024, 0.01, 2e-4, 1.0, (1.0, 1.0), scheme=2)
    assert int(lines[0]) == nt
    lv, co, _ = o.cells()
    assert np.array_equal(rows[:, 0].astype(int), lv)
    assert np.array_equal(rows[:, 1:3].astype(int), co)
    assert np.array_equal(rows[:, 3], o.cell_values())


@pytest.mark.gpu
@pytest.mark.parametrize("relative", [False, True])
def test_vector_demo_matches_oracle(tmp_path, relative):
    """make_vector_field<double, 2> through the C++ header: adaptation to both
    details, per-component Dirichlet values, upwind on the vector field;
    against the oracle's two-field restatement, bit for bit."""
    from advection_cases import centers
    from oracle.pyoracle import OracleSim

    exe = compile_demo(tmp_path, VSRC)
    out = os.path.join(str(tmp_path), "out.txt")
    subprocess.check_call([exe, out] + (["relative"] if relative else []))
    lines = open(out).read().split("\n")
    rows = np.array([[float(v) for v in l.split()] for l in lines[1:] if l.strip()])
    o = OracleSim(2, 3, 8, 1, 1, 1, 0.0)
    k1 = o.add_field(0.25)
    lv, co, _ = o.cells()
    c = centers(lv, co)
    x, y = c[:, 0], c[:, 1]
    o.set_cell_values(np.where((x - 0.3) * (x - 0.3) + (y - 0.3) * (y - 0.3) <= 0.2 * 0.2, 1.0, 0.0))
    o.set_cell_values_k(k1, np.where((x >= 0.5) & (x <= 0.7) & (y >= 0.4) & (y <= 0.6), 0.5, 0.0))
    dt = 0.5 / 256
    for _ in range(int(lines[0])):
        o.adapt_fields(1e-3, 1.0, 2, 0, relative_detail=relative)
        o.update_ghost_k(0)
        o.update_ghost_k(k1)
        o.upwind_k(0, (1.0, 0.5), dt)
        o.upwind_k(k1, (1.0, 0.5), dt)
    lv, co, _ = o.cells()
    assert np.array_equal(rows[:, 0].astype(int), lv)
    assert np.array_equal(rows[:, 1:3].astype(int), co)
    assert np.array_equal(rows[:, 3], o.cell_values())
    assert np.array_equal(rows[:, 4], o.cell_values_k(k1))


@pytest.mark.gpu
def test_demo_periodic_matches_oracle(tmp_path):
    """The demo on a mesh periodic along both axes (config.periodic(true) in
    the C++ header), against the oracle running the same loop."""
    from advection_cases import demo_time_loop, disc
    from oracle.pyoracle import OracleSim

    exe = compile_demo(tmp_path)
    out = os.path.join(str(tmp_path), "out.txt")
    subprocess.check_call([exe, "1", out, "periodic"])
    lines = open(out).read().split("\n")
    rows = np.array([[float(v) for v in l.split()] for l in lines[1:] if l.strip()])
    o = OracleSim(2, 4, 10, 1, 1, periodic=(True, True, False))
    lv, co, _ = o.cells()
    o.set_cell_values(disc(lv, co))
    o.adapt(2e-4, 1.0)
    nt = demo_time_loop(o, 0.5 / 1024, 0.01, 2e-4, 1.0, (1.0, 1.0))
    assert int(lines[0]) == nt
    lv, co, _ = o.cells()
    assert np.array_equal(rows[:, 0].astype(int), lv)
    assert np.array_equal(rows[:, 1:3].astype(int), co)
    assert np.array_equal(rows[:, 3], o.cell_values())


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["default", "refine_boundary"])
def test_demo_default_config_matches_oracle(tmp_path, mode):
    """The demo with samurai's default configuration, mra::make_mesh(box,
    mesh_config<2>().min_level(4).max_level(10)) without
    disable_minimal_ghost_width() (max_stencil_radius 2), and with
    samurai::args::refine_boundary, against the oracle running the same loop."""
    from advection_cases import demo_time_loop, disc
    from oracle.pyoracle import OracleSim

    exe = compile_demo(tmp_path)
    out = os.path.join(str(tmp_path), "out.txt")
    subprocess.check_call([exe, "1", out, mode])
    lines = open(out).read().split("\n")
    rows = np.array([[float(v) for v in l.split()] for l in lines[1:] if l.strip()])
    o = OracleSim(2, 4, 10, 2, 1)
    o.set_refine_boundary(mode == "refine_boundary")
    lv, co, _ = o.cells()
    o.set_cell_values(disc(lv, co))
    o.adapt(2e-4, 1.0)
    nt = demo_time_loop(o, 0.5 / 1024, 0.01, 2e-4, 1.0, (1.0, 1.0))
    assert int(lines[0]) == nt
    lv, co, _ = o.cells()
    assert np.array_equal(rows[:, 0].astype(int), lv)
    assert np.array_equal(rows[:, 1:3].astype(int), co)
    assert np.array_equal(rows[:, 3], o.cell_values())


@pytest.mark.gpu
def test_for_each_interval_through_the_header(tmp_path):
    """for_each_interval and u(level, i, j) of the C++ header after an
    adaptation: the oracle's leaf intervals and values."""
    from advection_cases import centers
    from oracle.pyoracle import OracleSim

    exe = compile_demo(tmp_path, ISRC)
    out = os.path.join(str(tmp_path), "out.txt")
    subprocess.check_call([exe, out])
    lines = [l.split() for l in open(out).read().split("\n") if l.strip()]
    o = OracleSim(2, 3, 7, 1, 1)
    lv, co, _ = o.cells()
    c = centers(lv, co)
    o.set_cell_values(np.where((c[:, 0] - 0.4) * (c[:, 0] - 0.4) + (c[:, 1] - 0.6) * (c[:, 1] - 0.6) < 0.04, 1.0, 0.0))
    o.adapt(1e-3, 1.0)
    ivs = [(int(l[1]), int(l[2]), int(l[3]), int(l[4])) for l in lines if l[0] == "I"]
    want = []
    for level in range(3, 8):
        want.extend((level,) + tuple(int(v) for v in r) for r in o.intervals("cells", level))
    assert ivs == want
    cells = np.array([[float(v) for v in l[1:]] for l in lines if l[0] == "C"])
    lv, co, _ = o.cells()
    assert np.array_equal(cells[:, 0].astype(int), lv) and np.array_equal(cells[:, 1:3].astype(int), co)
    assert np.array_equal(cells[:, 3], o.cell_values())


@pytest.mark.gpu
def test_fields_and_mesh_ids_through_the_header(tmp_path):
    """make_scalar_field with a value and with a function, u.fill,
    mesh.nb_cells(mesh_id) and for_each_cell / for_each_interval over
    mesh[mesh_id]: the oracle's counts and values."""
    from advection_cases import centers
    from oracle.pyoracle import OracleSim

    exe = compile_demo(tmp_path, FSRC)
    out = os.path.join(str(tmp_path), "out.txt")
    subprocess.check_call([exe, out])
    got = {l.split()[0]: float(l.split()[1]) for l in open(out).read().split("\n") if l.strip()}
    o = OracleSim(2, 2, 6, 1, 1)
    lv, co, _ = o.cells()
    c = centers(lv, co)
    x, y = c[:, 0], c[:, 1]
    o.set_cell_values(np.where((x >= 0.3) & (x <= 0.6) & (y >= 0.4) & (y <= 0.7), 1.0, 0.0))
    o.adapt(1e-3, 1.0)
    n_cells, n_ref = o.nb_cells(), o.nb_ref()

    def count(mid):
        return sum(int(r[1] - r[0]) for l in range(7) for r in o.intervals(mid, l))

    assert got["cells"] == n_cells and got["reference"] == n_ref
    for mid in ("cells_and_ghosts", "proj_cells", "union_cells"):
        assert got[mid] == count(mid), mid
    su = 0.0
    for v in o.cell_values():
        su += v
    assert got["sum_u"] == su
    assert got["sum_v"] == 2.5 * n_cells
    assert got["nref_walk"] == n_ref and got["nproj_walk"] == count("proj_cells")
    assert got["sum_fill"] == -n_cells
