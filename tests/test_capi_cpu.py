"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and
exports every function that include/samurai_gpu.h declares.  No compute call
is made here (there is no GPU)."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "samurai_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(sg_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["sg_mesh_create", "sg_field_create", "sg_adapt", "sg_update_ghost_mr", "sg_upwind", "sg_last_error"]:
        assert s in syms


def test_library_exports_all_declared_symbols():
    from samurai_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_no_cpu_fallback_without_gpu():
    import samurai_gb300 as sg
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(sg.SamuraiGpuError):
        sg.MRMesh(2, 2, 5)


def test_unit_box_only():
    import samurai_gb300 as sg
    with pytest.raises(sg.SamuraiGpuError):
        sg.Box([0, 0], [2, 1])


def test_minimal_ghost_width_rule():
    import samurai_gb300 as sg
    cfg = sg.mesh_config(2).min_level(2).max_level(5)
    assert cfg.parse_args() == 2  # mesh_config.hpp:388-393
    assert cfg.max_stencil_size(2).disable_minimal_ghost_width().parse_args() == 1


def test_batch_argument_checks():
    """sg_batch_create validates its arguments before touching a device."""
    import ctypes

    import samurai_gb300 as sg

    L = sg.lib()
    h = ctypes.c_void_p()
    arr = (ctypes.c_void_p * 1)()
    assert L.sg_batch_create(0, arr, arr, 1, ctypes.byref(h)) == 1
    assert b"n > 0" in L.sg_last_error()
    assert L.sg_batch_create(1, arr, arr, 1, ctypes.byref(h)) == 1
    assert b"two distinct fields" in L.sg_last_error()
    assert L.sg_batch_create(1, arr, arr, 0, ctypes.byref(h)) == 1
    assert L.sg_batch_step(None, None, None, None, None, 0, None) == 1
    assert L.sg_batch_synchronize(None) == 1
    assert L.sg_batch_autotune(None, None, None, None, None, 0, 3, None, None) == 1
    assert L.sg_batch_launch_shape(None, None, None) == 1
    assert L.sg_launch_shape(None, None, None, None, None, None, None, None) == 1
    assert L.sg_autotune(None, None, 1e-4, 2.0, None, 0.1, 0, 3, None, None) == 1


def test_mesh_create_rejects_unsupported_configurations():
    """sg_mesh_create checks its configuration before touching a device:
    dimension 2 or 3, 1 <= min_level <= max_level <= 23, stencil radius 1 or 2,
    prediction radius 0 or 1 (include/samurai_gpu.h)."""
    import ctypes

    import samurai_gb300 as sg

    L = sg.lib()
    h = ctypes.c_void_p()
    bad = [
        (1, 2, 5, 1, 1, 1),   # dimension
        (4, 2, 5, 1, 1, 1),
        (2, 0, 5, 1, 1, 1),   # min_level >= 1
        (2, 6, 5, 1, 1, 1),   # min_level <= max_level
        (2, 2, 24, 1, 1, 1),  # max_level <= 23
        (2, 2, 5, 3, 1, 1),   # stencil radius 1 or 2
        (2, 2, 5, 1, 2, 1),   # prediction radius 0 or 1
    ]
    for args in bad:
        assert L.sg_mesh_create(*args, ctypes.byref(h)) == 1, args
        assert L.sg_last_error()
    assert L.sg_mesh_create(2, 2, 5, 1, 1, 1, None) == 1
    # 3D levels whose bitmap sizes overflow 64-bit integers are refused before any device call
    for maxl in (16, 20, 23):
        assert L.sg_mesh_create(3, 2, maxl, 1, 1, 1, ctypes.byref(h)) == 3, maxl
        assert b"too fine" in L.sg_last_error()


def test_adjoint_argument_checks():
    import ctypes

    import samurai_gb300 as sg

    L = sg.lib()
    h = ctypes.c_void_p()
    assert L.sg_adjoint_create(None, 16, ctypes.byref(h)) == 1
    assert L.sg_adjoint_backward(None, None, None, None) == 1
    assert L.sg_adjoint_replay(None, None, None, None) == 1
    assert L.sg_adjoint_destroy(None) == 0


def test_vector_field_argument_checks():
    """make_vector_field / make_bc / make_MRAdapt on vector handles: malformed
    calls are rejected with SG_ERR_ARG before any device work."""
    import ctypes

    import samurai_gb300 as sg

    L = sg.lib()
    h = ctypes.c_void_p()
    assert L.sg_vector_field_create(None, b"v", 2, ctypes.byref(h)) == 1
    assert b"n_comp" in L.sg_last_error()
    assert L.sg_vector_field_component(None, 0, ctypes.byref(h)) == 1
    assert L.sg_vector_field_set_dirichlet(None, None) == 1
    assert L.sg_vector_field_swap(None, None) == 1
    assert L.sg_vector_adapt(None, 1e-3, 1.0, 0, None) == 1
    assert L.sg_vector_update_ghost_mr(None) == 1
    assert L.sg_vector_upwind(None, None, None, 0.1, 0) == 1
    assert L.sg_vector_field_download(None, None, 0) == 1
    assert L.sg_vector_field_destroy(None) == 0


def test_header_is_c99_and_a_c_client_links(tmp_path):
    """include/samurai_gpu.h is a C header (strict C99, no warnings) and a C
    program making the demo's loop through it links against the library"""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from samurai_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "abi_c_client")
    src = os.path.join(ROOT, "tests", "cpp", "abi_c_client.c")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I" + os.path.join(ROOT, "include"), src, "-o", exe,
                        lib, "-Wl,-rpath," + os.path.dirname(lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
