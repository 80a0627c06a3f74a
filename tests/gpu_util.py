"""Helpers shared by the GPU parity tests."""
import numpy as np

MESH_IDS = ["cells", "cells_and_ghosts", "proj_cells", "union_cells", "reference"]


def compare_meshes(gpu, ora, max_level, where=""):
    """Every MRMesh id, every level: identical intervals (canonical form)."""
    for mid in MESH_IDS:
        for level in range(0, max_level + 1):
            a = gpu.intervals(mid, level)
            b = ora.intervals(mid, level)
            assert a.shape == b.shape and np.array_equal(a, b), "%s: %s level %d differ (gpu %d / oracle %d intervals)" % (
                where, mid, level, len(a), len(b))


def compare_cells(gpu, ora, where=""):
    lg, cg, ig = gpu.cells()
    lo, co, io = ora.cells()
    assert np.array_equal(lg, lo) and np.array_equal(cg, co), where + ": leaf cells differ"
    assert np.array_equal(ig, io), where + ": storage indices differ"


def compare_fields(gpu, ora, where="", cells_only=False, rtol=0.0):
    """Bit-exact (rtol 0) on every reference entry the oracle defines; the
    oracle holds NaN where samurai's storage is indeterminate."""
    fg = gpu.field()
    fo = ora.field()
    assert fg.shape == fo.shape, where + ": reference sizes differ"
    if cells_only:
        _, _, idx = ora.cells()
        fg, fo = fg[idx], fo[idx]
    ok = ~np.isnan(fo)
    if rtol == 0.0:
        bad = np.flatnonzero(ok & (fg != fo))
        assert bad.size == 0, "%s: %d entries differ, first %s gpu=%r oracle=%r" % (
            where, bad.size, bad[:5], fg[bad[:5]], fo[bad[:5]])
    else:
        np.testing.assert_allclose(fg[ok], fo[ok], rtol=rtol, atol=0)
