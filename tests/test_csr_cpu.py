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
