"""SHA-256 digests of the oracle's state along the benchmark's full-size runs.

The 3D min_level 3 / max_level 9 workload (ball + 8 Gaussians, seed 2026) starts
from the uniform level-9 mesh: 134 M cells, minutes of oracle time and GBs of
host memory, too much for a test run.  The 2D min_level 4 / max_level 12
workload (16 squares + 16 Gaussians, seed 2026) is cheaper but the benchmark
steps it 25 times.  This script runs the oracle (the CPU restatement of
samurai's path, test infrastructure) through each run once and records, after
the initial adaptation and after every time step, a digest of the leaf cells and
their values in for_each_cell order:

    sha256(level as <i4 | coordinates as <i4, row per cell | values as <f8)

tests/test_gpu_fullsize.py recomputes the digests from the GPU's state: equal
digests mean bit-identical meshes and values.

The initial values are Gaussians and indicators evaluated by numpy, whose exp
differs in the last bit between x86-64 (its own vectorised exp) and aarch64
(the C library's), and the runs amplify such differences.  The digests are
therefore those of the machine architecture that generated them (recorded in
the file), and the test compares only on that architecture: the GB300 hosts,
aarch64, where the file was generated.

    python tests/golden/make_state_digests.py [--out FILE] [2d] [3d]     # default FILE: tests/golden/state_digests.json
"""
import hashlib
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from advection_cases import ball_3d, shapes_2d  # noqa: E402

OUT = os.path.join(HERE, "state_digests.json")

RUNS = {
    "2d": dict(dim=2, min_level=4, max_level=12, u0="shapes_2d(2026)", eps=1e-4, regularity=2.0, a=[1.0, 0.5], cfl=0.5, steps=25),
    "3d": dict(dim=3, min_level=3, max_level=9, u0="ball_3d(2026)", eps=1e-3, regularity=1.0, a=[1.0, 1.0, 1.0], cfl=0.3, steps=3),
}


def state_digest(level, coords, values):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(level, "<i4").tobytes())
    h.update(np.ascontiguousarray(coords, "<i4").tobytes())
    h.update(np.ascontiguousarray(values, "<f8").tobytes())
    return h.hexdigest()


def initial_function(run):
    return {"shapes_2d(2026)": shapes_2d(2026), "ball_3d(2026)": ball_3d(2026)}[run["u0"]]


def run_oracle(name):
    from oracle.pyoracle import OracleSim

    r = RUNS[name]
    o = OracleSim(r["dim"], r["min_level"], r["max_level"], 1, 1)
    lv, co, _ = o.cells()
    o.set_cell_values(initial_function(r)(lv, co))
    del lv, co
    t0 = time.time()
    passes = o.adapt(r["eps"], r["regularity"])
    out = {"run": r, "passes": [passes], "cells": [], "digests": []}

    def snap():
        lv, co, _ = o.cells()
        out["cells"].append(int(len(lv)))
        out["digests"].append(state_digest(lv, co, o.cell_values()))

    snap()
    print(name, "initial adaptation", round(time.time() - t0, 1), "s", out["cells"][-1], "cells", flush=True)
    dt = r["cfl"] / (1 << r["max_level"])
    for k in range(r["steps"]):
        out["passes"].append(o.adapt(r["eps"], r["regularity"]))
        o.update_ghost()
        o.upwind(r["a"], dt, 0)
        snap()
        print(name, "step", k + 1, round(time.time() - t0, 1), "s", out["cells"][-1], "cells", flush=True)
    return out


def main():
    argv = sys.argv[1:]
    out = OUT
    if "--out" in argv:
        k = argv.index("--out")
        out = argv[k + 1]
        del argv[k:k + 2]
    names = [a for a in argv if a in RUNS] or list(RUNS)
    data = json.load(open(out)) if os.path.exists(out) else {}
    for n in names:
        data[n] = run_oracle(n)
        data[n]["machine"] = platform.machine()
        json.dump(data, open(out, "w"), indent=1)


if __name__ == "__main__":
    main()
