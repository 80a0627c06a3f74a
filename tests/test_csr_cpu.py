"""The LevelCellArray layout written into restart files (samurai_gb300/csrc/
sg_csr.hpp, a streaming builder over the x-intervals) against the recursive
restatement of init_from_level_cell_list (level_cell_array.hpp:1005-1077) in
advection_cases.level_cell_array, on random 2D and 3D levels with empty rows,
empty planes and gaps."""
import os
import subprocess

import numpy as np
import pytest

from advection_cases import level_cell_array

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("csr") / "csr_tool")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", os.path.join(ROOT, "tests", "cpp", "csr_tool.cpp"), "-o", exe])
    return exe


def random_rows(rng, dim, n=12):
    occ = rng.random((n,) * dim) < rng.choice([0.05, 0.3, 0.7])
    rows, idx = [], 0
    keys = [(y,) for y in range(n)] if dim == 2 else [(z, y) for z in range(n) for y in range(n)]
    for key in keys:
        line = occ[key[0]] if dim == 2 else occ[key[0], key[1]]
        x = 0
        while x < n:
            if line[x]:
                s = x
                while x < n and line[x]:
                    x += 1
                rows.append([s - 3, x - 3, key[-1] - 5] + ([key[0] - 2] if dim == 3 else []) + [idx - (s - 3)])
                idx += x - s
            else:
                x += 1
    return rows


@pytest.mark.parametrize("dim", [2, 3])
def test_streaming_builder_matches_the_restatement(tool, dim):
    rng = np.random.default_rng(7 + dim)
    for _ in range(60):
        rows = random_rows(rng, dim)
        text = "%d %d\n" % (dim, len(rows)) + "\n".join(" ".join(map(str, r)) for r in rows)
        out = subprocess.run([tool], input=text.encode(), capture_output=True, check=True).stdout.decode().split("\n")
        ivs, offs = level_cell_array(rows, dim)
        want = ["iv%d" % d + "".join(" %d,%d,%d" % t for t in ivs[d]) for d in range(dim)]
        want += ["off%d" % d + "".join(" %d" % v for v in offs[d]) for d in range(dim - 1)]
        assert out[:len(want)] == want


def rows_in_box(rng, dim, n=12):
    """random_rows shifted into the level-4 box [0, 16)"""
    rows = random_rows(rng, dim, n)
    out = []
    for r in rows:
        s, e, y = r[0] + 3, r[1] + 3, r[2] + 5
        key = [y] + ([r[3] + 2] if dim == 3 else [])
        out.append([s, e] + key + [r[-1] - 3])
    return out


@pytest.mark.parametrize("dim", [2, 3])
def test_decode_inverts_the_builder(tool, dim):
    """decode_csr (what sg_load walks) gives back the cells of the rows the
    layout was built from, in for_each_cell order"""
    rng = np.random.default_rng(11 + dim)
    for _ in range(40):
        rows = rows_in_box(rng, dim)
        text = "%d %d\n" % (dim, len(rows)) + "\n".join(" ".join(map(str, r)) for r in rows)
        out = subprocess.run([tool, "decode", "4"], input=text.encode(), capture_output=True, check=True).stdout.decode().split("\n")
        want = []
        for r in rows:
            for x in range(r[0], r[1]):
                want.append(",".join(map(str, [x] + r[2:2 + dim - 1])))
        assert out[dim + dim - 1] == "dec 0"
        assert out[dim + dim].split()[1:] == want


@pytest.fixture(scope="module")
def fuzz_tool(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("csrfuzz") / "csr_tool")
    src = os.path.join(ROOT, "tests", "cpp", "csr_tool.cpp")
    san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-g"]
    if subprocess.run(["g++", "-std=c++17", "-O1"] + san + [src, "-o", exe], capture_output=True).returncode != 0:
        subprocess.check_call(["g++", "-std=c++17", "-O1", src, "-o", exe])
    return exe


@pytest.mark.parametrize("dim,seed", [(2, 1), (2, 2), (3, 3), (3, 4)])
def test_decode_refuses_corrupted_layouts(fuzz_tool, dim, seed):
    """restart layouts come from files: overwritten interval bounds and
    indices and offsets entries are refused (outside the box or
    inconsistent), never read outside the arrays"""
    rng = np.random.default_rng(100 + seed)
    rows = rows_in_box(rng, dim)
    while len(rows) < 4:
        rows = rows_in_box(rng, dim)
    text = "%d %d\n" % (dim, len(rows)) + "\n".join(" ".join(map(str, r)) for r in rows)
    r = subprocess.run([fuzz_tool, "fuzz", "4", str(seed), "3000"], input=text.encode(), capture_output=True, timeout=300)
    assert r.returncode == 0, r.stderr.decode()[-2000:]
    ok, outside, inconsistent = (int(v) for v in r.stdout.split())
    assert ok + outside + inconsistent == 3000 and outside > 0 and inconsistent > 0


def decode_raw(tool, level, dim, ivs, offs):
    text = "%d\n" % dim
    for d in range(dim):
        text += "%d\n" % len(ivs[d]) + "".join("%d %d %d\n" % t for t in ivs[d])
    for d in range(dim - 1):
        text += "%d\n" % len(offs[d]) + "".join("%d\n" % v for v in offs[d])
    out = subprocess.run([tool, "raw", str(level)], input=text.encode(), capture_output=True, check=True, timeout=60).stdout.split()
    return int(out[1]), int(out[2])


def test_decode_refuses_rows_sent_to_the_same_intervals(tool):
    """offsets that point many rows at one x-interval would make the walk repeat
    its cells without bound (a level-20 row repeated 1000 times is 2^30 cells);
    the layout is refused when an interval is reached a second time, so at most
    the cells of its first visit were appended"""
    level = 20
    full = [(0, 1 << level, 0)]
    # 1000 one-row y-intervals, each sent to offsets slot 0 (index = -y): the same full x-row every time
    ys = [(y, y + 1, -y) for y in range(1000)]
    assert decode_raw(tool, level, 2, [full, ys], [[0, 1]]) == (2, 1 << level)
    # 3D: many z-planes sent to the same y-interval
    zs = [(z, z + 1, -z) for z in range(60)]
    assert decode_raw(tool, 6, 3, [[(0, 64, 0)], [(0, 1, 0)], zs], [[0, 1], [0, 1]]) == (2, 64)
    # the one-row layouts themselves are accepted
    assert decode_raw(tool, level, 2, [full, [(5, 6, -5)]], [[0, 1]]) == (0, 1 << level)
    assert decode_raw(tool, 6, 3, [[(0, 64, 0)], [(0, 1, 0)], [(3, 4, -3)]], [[0, 1], [0, 1]]) == (0, 64)
