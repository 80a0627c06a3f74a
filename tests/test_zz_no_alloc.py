"""sg_field_download_noalloc, the entry point that allocates nothing.

A caller that cannot let this library allocate device memory (its GPU memory
is reserved by another allocator, or its loop must not pay for an allocation)
reads u.array() through this variant of sg_field_download: the gather kernel
writes into a static device array instead of a cudaMalloc'd staging buffer.
Through the C ABI it must return exactly what sg_field_download returns, on
consecutive calls, and refuse a mesh larger than the array (2^21 reference
cells).  The file is named to be collected last.
"""
import ctypes
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SG_ERR_CAPACITY = 3


def _api():
    from samurai_gb300 import build

    build.build()
    import samurai_gb300 as sg

    lib = sg.lib()
    lib.sg_field_download_noalloc.restype = ctypes.c_int
    lib.sg_field_download_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong]
    return sg, lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_noalloc_download_matches_download_on_consecutive_calls():
    sg, lib = _api()
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from advection_cases import shapes_2d

    sim = sg.AdvectionSim(2, 3, 9)
    lv, co, _ = sim.cells()
    sim.set_cell_values(shapes_2d(11, 4, 4)(lv, co))
    dt = 0.5 / (1 << 9)
    outputs = []
    for _ in range(2):
        sim.adapt(1e-4, 2.0)
        sim.update_ghost()
        sim.upwind([1.0, 0.5], dt)
        n = sim.nb_ref()
        expected = np.empty(n)
        assert lib.sg_field_download(sim.u.h, _ptr(expected), n) == 0
        for _ in range(2):  # two calls in a row on the same state
            got = np.full(n, np.nan)
            status = lib.sg_field_download_noalloc(sim.u.h, _ptr(got), n)
            assert status == 0, lib.sg_last_error().decode()
            assert np.array_equal(got, expected)  # bit-identical, as every parity test here
        outputs.append(got)
    # the second step's state differs from the first one's (its mesh or its values), so the shared array held
    # other contents when the second step's calls rewrote it
    assert outputs[0].shape != outputs[1].shape or not np.array_equal(outputs[0], outputs[1])


def test_noalloc_download_rejects_meshes_beyond_its_array():
    sg, lib = _api()
    mesh = sg.MRMesh(2, 1, 11)  # uniform at level 11: 2^22 reference cells
    u = sg.make_scalar_field("u", mesh)
    n = mesh.nb_cells("reference")
    assert n > (1 << 21)
    out = np.empty(n)
    assert lib.sg_field_download_noalloc(u.h, _ptr(out), n) == SG_ERR_CAPACITY
    assert "2^21" in lib.sg_last_error().decode()
