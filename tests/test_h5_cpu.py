"""The HDF5 layer (samurai_gb300/csrc/sg_h5.hpp) without a GPU: a file written
by the writer is decoded identically by the library's reader and by the
independent pure-Python reader of tests/h5lite.py (scalars, 2-D arrays,
signed and unsigned integers, binary64, samurai's Interval compound, a group
spread over several symbol-table nodes, an empty dataset), and corrupted
files are refused without reads outside the buffer."""
import os
import subprocess

import numpy as np
import pytest

from h5lite import H5

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("h5") / "h5_tool")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", os.path.join(ROOT, "tests", "cpp", "h5_tool.cpp"), "-o", exe])
    return exe


def read_with_tool(tool, path, name):
    out = subprocess.check_output([tool, "read", path, name]).decode().split("\n")
    head = [int(x) for x in out[0].split()]
    return head, [l for l in out[1:] if l]


def test_writer_reader_roundtrip(tool, tmp_path):
    f = str(tmp_path / "t.h5")
    subprocess.check_call([tool, "write", f])
    h = H5(f)
    assert h.keys() == ["empty", "many", "mesh", "n_process"]
    assert h.keys("/mesh") == ["connectivity", "fields", "level", "points"]
    assert len(h.keys("/many")) == 21
    assert int(h.read("/n_process")) == 1
    pts = h.read("/mesh/points")
    assert pts.shape == (4, 3) and pts[3, 0] == -1.5e300 and pts[3, 2] == 1e-300
    assert h.read("/mesh/connectivity").tolist() == [[0, 1, 2, 3], [3, 2, 1, 0]]
    assert h.read("/mesh/fields/signed").tolist() == [-5, 7, -9000000000]
    assert h.read("/mesh/fields/small").tolist() == [-1, 2147483647]
    iv = h.read("/mesh/level/4/dim/0/intervals/data")
    assert iv.dtype.names == ("start", "end", "step", "index") and iv.dtype.itemsize == 24
    assert [tuple(int(v) for v in r) for r in iv] == [(-3, 5, 1, 17), (8, 9, 1, -8)]
    for k in range(21):
        assert float(h.read("/many/m%d" % k)) == k * 0.5
    assert h.read("/empty").shape == (0,)

    head, vals = read_with_tool(tool, f, "/mesh/points")
    assert head == [1, 8, 0, 4, 3] and [float(v) for v in vals] == pts.reshape(-1).tolist()
    head, vals = read_with_tool(tool, f, "/mesh/fields/signed")
    assert head == [0, 8, 1, 3] and vals == ["-5", "7", "-9000000000"]
    head, vals = read_with_tool(tool, f, "/mesh/level/4/dim/0/intervals/data")
    assert head[:2] == [6, 24] and vals == ["-3 5 1 17", "8 9 1 -8"]
    head, vals = read_with_tool(tool, f, "/many/m20")
    assert head == [1, 8, 0] and vals == ["10"]
    assert subprocess.check_output([tool, "exists", f, "/many/m7"]).strip() == b"1"
    assert subprocess.check_output([tool, "exists", f, "/many/m77"]).strip() == b"0"
    assert subprocess.run([tool, "read", f, "/nothing"], capture_output=True).returncode == 1
    r = subprocess.run([tool, "toomany", str(tmp_path / "big.h5")], capture_output=True)
    assert r.returncode == 3 and b"256 members" in r.stderr


@pytest.fixture(scope="module")
def fuzz_tool(tmp_path_factory):
    """the same tool under the address and undefined-behaviour sanitizers
    (a plain build where the compiler has no sanitizer runtime)"""
    exe = str(tmp_path_factory.mktemp("h5fuzz") / "h5_tool")
    src = os.path.join(ROOT, "tests", "cpp", "h5_tool.cpp")
    san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-g"]
    if subprocess.run(["g++", "-std=c++17", "-O1"] + san + [src, "-o", exe], capture_output=True).returncode != 0:
        subprocess.check_call(["g++", "-std=c++17", "-O1", src, "-o", exe])
    return exe


@pytest.mark.parametrize("seed", range(1, 9))
def test_reader_refuses_corrupted_files(fuzz_tool, tmp_path, seed):
    """restart files come from users: truncated files, flipped bits and
    overwritten offsets, sizes and counts make the reader return an error
    (or a consistent array), never read outside the file"""
    f = str(tmp_path / "t.h5")
    subprocess.check_call([fuzz_tool, "write", f])
    r = subprocess.run([fuzz_tool, "fuzz", f, str(seed), "4000"], capture_output=True, timeout=300)
    assert r.returncode == 0, r.stderr.decode()[-2000:]
    opened, ok, refused = (int(v) for v in r.stdout.split())
    assert opened > 3000 and ok > 0 and refused > 0


def test_io_argument_checks():
    import ctypes

    import samurai_gb300 as sg

    L = sg.lib()
    h = ctypes.c_void_p()
    assert L.sg_io_create(ctypes.byref(h)) == 0
    assert L.sg_io_add_field(h, None) == 1
    assert L.sg_save(b"", b"x", None, h) == 1
    assert L.sg_dump(b"", None, None, h) == 1
    assert L.sg_load(b"", b"x", None, h) == 1
    d, lo, hi = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert L.sg_restart_levels(b"", b"no_such_file_here", ctypes.byref(d), ctypes.byref(lo), ctypes.byref(hi)) == 5
    assert L.sg_io_destroy(h) == 0
