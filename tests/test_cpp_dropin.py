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
GOLD = os.path.join(ROOT, "tests", "golden")


def compile_demo(tmp_path):
    from samurai_gb300 import build

    lib = build.build()
    exe = os.path.join(str(tmp_path), "advection_2d")
    cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), SRC, "-L" + os.path.dirname(lib), "-lsamurai_gpu",
           "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    subprocess.check_call(cmd)
    return exe


def test_demo_compiles(tmp_path):
    exe = compile_demo(tmp_path)
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
