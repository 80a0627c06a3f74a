"""GB300-native MR advection path with samurai's API names.

This package is the Python host side over the C ABI of libsamurai_gpu.so
(include/samurai_gpu.h).  It mirrors the calls a samurai user program makes
for the multiresolution advection path:

    cfg  = mesh_config(2).min_level(4).max_level(10).max_stencil_size(2).disable_minimal_ghost_width()
    mesh = mra.make_mesh(Box([0, 0], [1, 1]), cfg)        # mr/mesh.hpp:511-518
    u    = make_scalar_field("u", mesh)                    # field/scalar_field.hpp:173-216
    make_bc(Dirichlet(1), u, 0.)                           # bc/bc.hpp:786-800
    MRadaptation = make_MRAdapt(u)                         # mr/adapt.hpp:391-397
    MRadaptation(mra_config().epsilon(2e-4))               # mr/adapt.hpp:147-195
    update_ghost_mr(u)                                     # algorithm/update_ghost_mr.hpp:261-270
    unp1.assign_upwind(u, a, dt)                           # unp1 = u - dt * upwind(a, u)
    swap(u, unp1)                                          # std::swap(u.array(), unp1.array())

Everything that computes runs as sm_103a CUDA kernels; there is no CPU
fallback, and a missing or unloadable library raises at first use.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBPATH = os.path.join(_HERE, "libsamurai_gpu.so")
_lib = None

SG_CELLS, SG_CELLS_AND_GHOSTS, SG_PROJ_CELLS, SG_UNION_CELLS, SG_REFERENCE = range(5)
MESH_IDS = {"cells": 0, "cells_and_ghosts": 1, "proj_cells": 2, "union_cells": 3, "reference": 4, "all_cells": 4}
UPWIND_OP, README, CONVECTION = 0, 1, 2


class SamuraiGpuError(RuntimeError):
    pass


def library_path():
    return _LIBPATH


def lib():
    """Load libsamurai_gpu.so (built in-tree by samurai_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIBPATH):
        raise SamuraiGpuError("libsamurai_gpu.so is not built; run `python -m samurai_gb300.build` (there is no CPU fallback)")
    L = ctypes.CDLL(_LIBPATH)
    vp, i, d, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
    pi, pl = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong)
    sig = {
        "sg_last_error": (ctypes.c_char_p, []),
        "sg_version": (i, [pi, pi]),
        "sg_mesh_create": (i, [i, i, i, i, i, i, ctypes.POINTER(vp)]),
        "sg_mesh_create_periodic": (i, [i, i, i, i, i, i, vp, ctypes.POINTER(vp)]),
        "sg_mesh_destroy": (i, [vp]),
        "sg_mesh_counts": (i, [vp, pl, pl]),
        "sg_mesh_get_cells": (i, [vp, vp, vp, vp, ll]),
        "sg_mesh_count_intervals": (i, [vp, i, i, pl]),
        "sg_mesh_get_intervals": (i, [vp, i, i, vp, ll]),
        "sg_mesh_set_cells": (i, [vp, ll, vp, vp]),
        "sg_mesh_stream": (i, [vp, ctypes.POINTER(vp)]),
        "sg_mesh_synchronize": (i, [vp]),
        "sg_mesh_launch_count": (i, [vp, i, pl]),
        "sg_mesh_version": (i, [vp, ctypes.POINTER(ctypes.c_ulonglong)]),
        "sg_timers_enable": (i, [vp, i]),
        "sg_timers_get": (i, [vp, i, ctypes.POINTER(d), pl]),
        "sg_timers_reset": (i, [vp]),
        "sg_kernel_trace": (i, [vp, i]),
        "sg_mesh_set_refine_boundary": (i, [vp, i]),
        "sg_mesh_set_adapt_graph": (i, [vp, i]),
        "sg_kernel_trace_read": (i, [vp, i, ctypes.POINTER(ctypes.c_char_p), pl, ctypes.POINTER(d), pi]),
        "sg_device_fp64_rate": (i, [ctypes.POINTER(d)]),
        "sg_field_create": (i, [vp, ctypes.c_char_p, ctypes.POINTER(vp)]),
        "sg_field_destroy": (i, [vp]),
        "sg_field_set_dirichlet": (i, [vp, d]),
        "sg_field_upload": (i, [vp, vp, ll]),
        "sg_field_download": (i, [vp, vp, ll]),
        "sg_field_download_noalloc": (i, [vp, vp, ll]),
        "sg_field_upload_device": (i, [vp, vp, ll]),
        "sg_field_download_device": (i, [vp, vp, ll]),
        "sg_field_set_cells": (i, [vp, vp, ll]),
        "sg_field_get_cells": (i, [vp, vp, ll]),
        "sg_field_swap": (i, [vp, vp]),
        "sg_field_fill": (i, [vp, d]),
        "sg_adapt": (i, [vp, d, d, pi]),
        "sg_harten": (i, [vp, i, d, d, pi]),
        "sg_adapt_ex": (i, [vp, d, d, i, pi]),
        "sg_harten_ex": (i, [vp, i, d, d, i, pi]),
        "sg_adapt_fields": (i, [i, vp, i, vp, d, d, i, pi]),
        "sg_update_ghost_mr_fields": (i, [i, vp]),
        "sg_update_ghost_mr": (i, [vp]),
        "sg_upwind": (i, [vp, vp, vp, d, i]),
        "sg_step": (i, [vp, vp, d, d, vp, d, i, pi]),
        "sg_autotune": (i, [vp, vp, d, d, vp, d, i, i, ctypes.POINTER(d), ctypes.POINTER(d)]),
        "sg_launch_shape": (i, [vp, pi, pl, pl, pl, pl, pi, pi]),
        "sg_detail_download": (i, [vp, vp, ll]),
        "sg_tag_download": (i, [vp, vp, ll]),
        "sg_batch_create": (i, [i, vp, vp, i, ctypes.POINTER(vp)]),
        "sg_batch_destroy": (i, [vp]),
        "sg_batch_size": (i, [vp, pi]),
        "sg_batch_adapt": (i, [vp, vp, vp, vp]),
        "sg_batch_update_ghost_mr": (i, [vp]),
        "sg_batch_upwind": (i, [vp, vp, vp, i]),
        "sg_batch_swap": (i, [vp]),
        "sg_batch_step": (i, [vp, vp, vp, vp, vp, i, vp]),
        "sg_batch_synchronize": (i, [vp]),
        "sg_batch_autotune": (i, [vp, vp, vp, vp, vp, i, i, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
        "sg_batch_launch_shape": (i, [vp, pl, pi]),
        "sg_adjoint_create": (i, [vp, i, ctypes.POINTER(vp)]),
        "sg_adjoint_destroy": (i, [vp]),
        "sg_adjoint_counts": (i, [vp, pl, pl, pi]),
        "sg_adjoint_cells": (i, [vp, i, vp, vp, ll]),
        "sg_adjoint_record": (i, [vp, vp, i, d, d, vp, d, i, pl]),
        "sg_adjoint_final": (i, [vp, vp, ll]),
        "sg_adjoint_replay": (i, [vp, vp, vp, vp]),
        "sg_adjoint_backward": (i, [vp, vp, vp, vp]),
        "sg_vector_field_create": (i, [vp, ctypes.c_char_p, i, ctypes.POINTER(vp)]),
        "sg_vector_field_destroy": (i, [vp]),
        "sg_vector_field_n_comp": (i, [vp, pi]),
        "sg_vector_field_component": (i, [vp, i, ctypes.POINTER(vp)]),
        "sg_vector_field_set_dirichlet": (i, [vp, vp]),
        "sg_vector_field_upload": (i, [vp, vp, ll]),
        "sg_vector_field_download": (i, [vp, vp, ll]),
        "sg_vector_field_set_cells": (i, [vp, vp, ll]),
        "sg_vector_field_get_cells": (i, [vp, vp, ll]),
        "sg_vector_field_swap": (i, [vp, vp]),
        "sg_vector_adapt": (i, [vp, d, d, i, pi]),
        "sg_vector_update_ghost_mr": (i, [vp]),
        "sg_vector_upwind": (i, [vp, vp, vp, d, i]),
        "sg_io_create": (i, [ctypes.POINTER(vp)]),
        "sg_io_destroy": (i, [vp]),
        "sg_io_add_field": (i, [vp, vp]),
        "sg_io_add_vector_field": (i, [vp, vp]),
        "sg_save": (i, [ctypes.c_char_p, ctypes.c_char_p, vp, vp]),
        "sg_dump": (i, [ctypes.c_char_p, ctypes.c_char_p, vp, vp]),
        "sg_restart_levels": (i, [ctypes.c_char_p, ctypes.c_char_p, pi, pi, pi]),
        "sg_load": (i, [ctypes.c_char_p, ctypes.c_char_p, vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(status, what):
    if status != 0:
        msg = lib().sg_last_error().decode(errors="replace")
        raise SamuraiGpuError("%s failed (status %d): %s" % (what, status, msg))


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


# ---------------------------------------------------------------- configs
class Box:
    """samurai::Box<double, dim> (box.hpp); only the unit box is supported."""

    def __init__(self, min_corner, max_corner):
        self.min_corner = [float(v) for v in min_corner]
        self.max_corner = [float(v) for v in max_corner]
        if any(v != 0.0 for v in self.min_corner) or any(v != 1.0 for v in self.max_corner):
            raise SamuraiGpuError("only the unit box [0,1]^dim is supported")

    @property
    def dim(self):
        return len(self.min_corner)


class mesh_config:
    """samurai::mesh_config<dim, prediction_stencil_radius> (mesh_config.hpp:16-433)."""

    def __init__(self, dim, prediction_stencil_radius=1):
        self.dim = dim
        self.prediction_stencil_radius = prediction_stencil_radius
        self._min_level = 0
        self._max_level = 6
        self._max_stencil_radius = 1
        self._graduation_width = 1
        self._disable_minimal_ghost_width = False
        self._periodic = [False] * dim

    def periodic(self, p=None):
        """periodic(bool) fills every axis, periodic([..]) sets them one by one, periodic() reads them
        (mesh_config.hpp:279-331)"""
        if p is None:
            return list(self._periodic)
        if isinstance(p, (bool, int)):
            self._periodic = [bool(p)] * self.dim
        else:
            if len(p) != self.dim:
                raise ValueError("one periodicity flag per axis")
            self._periodic = [bool(v) for v in p]
        return self

    def min_level(self, l):
        self._min_level = l
        return self

    def max_level(self, l):
        self._max_level = l
        return self

    def max_stencil_radius(self, r):
        self._max_stencil_radius = r
        return self

    def max_stencil_size(self, s):
        self._max_stencil_radius = s // 2 + (s % 2)
        return self

    def graduation_width(self, w):
        self._graduation_width = w
        return self

    def disable_minimal_ghost_width(self):
        self._disable_minimal_ghost_width = True
        return self

    def parse_args(self):
        """mesh_config::parse_args without command-line overrides (mesh_config.hpp:358-396)."""
        if self._max_level < self._min_level:
            raise ValueError("Max level must be greater than min level.")
        r = self._max_stencil_radius
        if not self._disable_minimal_ghost_width:
            r = max(r, 2)
        return r


class mra_config:
    """samurai::mra_config (mr/config.hpp:10-67)."""

    def __init__(self):
        self._epsilon = 1e-4
        self._regularity = 1.0
        self._relative_detail = False

    def epsilon(self, v=None):
        if v is None:
            return self._epsilon
        self._epsilon = v
        return self

    def regularity(self, v=None):
        if v is None:
            return self._regularity
        self._regularity = v
        return self

    def relative_detail(self, v=None):
        if v is None:
            return self._relative_detail
        self._relative_detail = bool(v)
        return self


# ------------------------------------------------------------------ mesh
class MRMesh:
    """samurai::MRMesh on the unit box (mr/mesh.hpp:74-211), device resident."""

    def __init__(self, dim, min_level, max_level, max_stencil_radius=1, prediction_radius=1, graduation_width=1, periodic=None):
        self.dim = dim
        self._min_level = min_level
        self._max_level = max_level
        self.max_stencil_radius = max_stencil_radius
        self.prediction_radius = prediction_radius
        self.graduation_width = graduation_width
        self.periodic = [bool(p) for p in periodic][:dim] if periodic is not None else [False] * dim
        h = ctypes.c_void_p()
        per = (ctypes.c_int * 3)(*([int(p) for p in self.periodic] + [0] * (3 - dim)))
        _check(lib().sg_mesh_create_periodic(dim, min_level, max_level, max_stencil_radius, prediction_radius, graduation_width, per,
                                             ctypes.byref(h)), "sg_mesh_create")
        self.h = h

    @classmethod
    def from_box(cls, box, min_level, max_level):
        """Deprecated samurai constructor MRMesh<MRConfig<dim>>(box, min, max) (mr/mesh.hpp:166-181)."""
        return cls(box.dim, min_level, max_level)

    def __del__(self):
        if getattr(self, "h", None):
            try:
                lib().sg_mesh_destroy(self.h)
            except Exception:
                pass
            self.h = None

    def min_level(self):
        return self._min_level

    def max_level(self):
        return self._max_level

    def cell_length(self, level):
        """cell_length(1, level) (cell.hpp:17-20)"""
        return 1.0 / (1 << level)

    def min_cell_length(self):
        return self.cell_length(self._max_level)

    def counts(self):
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        _check(lib().sg_mesh_counts(self.h, ctypes.byref(a), ctypes.byref(b)), "sg_mesh_counts")
        return a.value, b.value

    def nb_cells(self, mesh_id="reference"):
        nc, nr = self.counts()
        return nr if MESH_IDS.get(mesh_id, mesh_id) == SG_REFERENCE else nc

    def cells(self):
        """for_each_cell order: (level, coords, storage index)"""
        n, _ = self.counts()
        level = np.empty(n, np.int32)
        coords = np.empty((n, self.dim), np.int32)
        index = np.empty(n, np.int64)
        _check(lib().sg_mesh_get_cells(self.h, _ptr(level), _ptr(coords), _ptr(index), n), "sg_mesh_get_cells")
        return level, coords, index

    def intervals(self, mesh_id, level, with_index=False):
        mid = MESH_IDS[mesh_id] if isinstance(mesh_id, str) else mesh_id
        n = ctypes.c_longlong()
        _check(lib().sg_mesh_count_intervals(self.h, mid, level, ctypes.byref(n)), "sg_mesh_count_intervals")
        out = np.empty((n.value, self.dim + 2), np.int64)
        _check(lib().sg_mesh_get_intervals(self.h, mid, level, _ptr(out), n.value), "sg_mesh_get_intervals")
        return out if with_index else out[:, : self.dim + 1].astype(np.int32)

    def version(self):
        """changes whenever the cells change (adaptation, set_cells, load)"""
        v = ctypes.c_ulonglong()
        _check(lib().sg_mesh_version(self.h, ctypes.byref(v)), "sg_mesh_version")
        return v.value

    def find(self, level, i, *yz):
        """storage index of cell (i, yz...) of the reference mesh at a level, -1 if absent
        (get_index, algorithm.hpp:391-467)"""
        v = self.version()
        if getattr(self, "_rows_version", None) != v:
            rows = {}
            for l in range(self._max_level + 1):
                for r in self.intervals("reference", l, with_index=True):
                    rows.setdefault((l,) + tuple(int(t) for t in r[2:self.dim + 1]), []).append((int(r[0]), int(r[1]), int(r[self.dim + 1])))
            self._rows, self._rows_version = rows, v
        for s0, e0, idx in self._rows.get((int(level),) + tuple(int(t) for t in yz), ()):
            if s0 <= i < e0:
                return idx + int(i)
        return -1

    def set_cells(self, level, coords):
        level = np.ascontiguousarray(level, np.int32)
        coords = np.ascontiguousarray(coords, np.int32)
        _check(lib().sg_mesh_set_cells(self.h, len(level), _ptr(level), _ptr(coords)), "sg_mesh_set_cells")

    def stream(self):
        s = ctypes.c_void_p()
        _check(lib().sg_mesh_stream(self.h, ctypes.byref(s)), "sg_mesh_stream")
        return s.value

    def synchronize(self):
        _check(lib().sg_mesh_synchronize(self.h), "sg_mesh_synchronize")

    TIMER_NAMES = ["mesh adaptation", "ghost update", "detail computation", "tag cells", "tag finalization", "mesh update",
                   "make_graduation", "mesh construction", "fields update", "field expressions"]

    def timers(self, enable=None, reset=False):
        """samurai's named timers as {name: (ms, calls)}; enable/reset on request"""
        if enable is not None:
            _check(lib().sg_timers_enable(self.h, 1 if enable else 0), "sg_timers_enable")
        if reset:
            _check(lib().sg_timers_reset(self.h), "sg_timers_reset")
        out = {}
        for k, name in enumerate(self.TIMER_NAMES):
            ms, n = ctypes.c_double(), ctypes.c_longlong()
            _check(lib().sg_timers_get(self.h, k, ctypes.byref(ms), ctypes.byref(n)), "sg_timers_get")
            out[name] = (ms.value, n.value)
        return out

    def launch_shape(self):
        """{block, max_blocks, fuse_mesh_words, fuse_field_words, fuse_max_words, graphed_adapt, level_pairs} of this mesh's launches"""
        b, mb, fm, ff, fx = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        gr, lp = ctypes.c_int(), ctypes.c_int()
        _check(lib().sg_launch_shape(self.h, ctypes.byref(b), ctypes.byref(mb), ctypes.byref(fm), ctypes.byref(ff), ctypes.byref(fx),
                                     ctypes.byref(gr), ctypes.byref(lp)), "sg_launch_shape")
        return {"block": b.value, "max_blocks": mb.value, "fuse_mesh_words": fm.value, "fuse_field_words": ff.value, "fuse_max_words": fx.value,
                "graphed_adapt": bool(gr.value), "level_pairs": bool(lp.value)}

    def set_adapt_graph(self, enable):
        """each adaptation as one captured graph with conditional nodes (True) or pass by pass (False, the default)"""
        _check(lib().sg_mesh_set_adapt_graph(self.h, 1 if enable else 0), "sg_mesh_set_adapt_graph")

    def set_refine_boundary(self, enable):
        """samurai's --refine-boundary (args::refine_boundary) for this mesh's adaptations"""
        _check(lib().sg_mesh_set_refine_boundary(self.h, 1 if enable else 0), "sg_mesh_set_refine_boundary")

    def kernel_trace(self, enable):
        """start (True) or stop (False) the per-launch kernel trace; stopping
        returns (rows, valid), rows = [(kernel, launches, ms)] in order of first
        launch; valid is False when a captured sequence ran twice in the window"""
        _check(lib().sg_kernel_trace(self.h, 1 if enable else 0), "sg_kernel_trace")
        if enable:
            return None
        rows, valid = [], True
        k = 0
        while True:
            name, n, ms, ok = ctypes.c_char_p(), ctypes.c_longlong(), ctypes.c_double(), ctypes.c_int()
            st = lib().sg_kernel_trace_read(self.h, k, ctypes.byref(name), ctypes.byref(n), ctypes.byref(ms), ctypes.byref(ok))
            if st == 5:  # SG_ERR_NOTFOUND: past the last entry
                break
            _check(st, "sg_kernel_trace_read")
            rows.append((name.value.decode(), n.value, ms.value))
            valid = valid and bool(ok.value)
            k += 1
        return rows, valid

    def launch_count(self, reset=False):
        n = ctypes.c_longlong()
        _check(lib().sg_mesh_launch_count(self.h, 1 if reset else 0, ctypes.byref(n)), "sg_mesh_launch_count")
        return n.value


class mra:
    @staticmethod
    def make_mesh(box, cfg):
        """samurai::mra::make_mesh(box, cfg) (mr/mesh.hpp:511-518): uniform at max_level"""
        if box.dim != cfg.dim:
            raise ValueError("box and config dimensions differ")
        r = cfg.parse_args()
        return MRMesh(cfg.dim, cfg._min_level, cfg._max_level, r, cfg.prediction_stencil_radius, cfg._graduation_width,
                      periodic=cfg._periodic)


# ----------------------------------------------------------------- fields
class ScalarField:
    """samurai::ScalarField<MRMesh, double> (field/scalar_field.hpp:77-216)."""

    n_comp = 1

    def __init__(self, name, mesh, _handle=None):
        self.name = name
        self.mesh = mesh
        self._owner = _handle is None
        if _handle is None:
            h = ctypes.c_void_p()
            _check(lib().sg_field_create(mesh.h, name.encode(), ctypes.byref(h)), "sg_field_create")
        else:
            h = _handle  # a component of a vector field, owned by it
        self.h = h

    def components(self):
        return [self]

    def fill(self, value):
        """u.fill(value) (field/access_base.hpp:63-66): every reference cell"""
        _check(lib().sg_field_fill(self.h, float(value)), "sg_field_fill")

    def __call__(self, level, i, *yz):
        """u(level, i, j[, k]): the value of a reference cell (host copy)"""
        e = self.mesh.find(level, i, *yz)
        if e < 0:
            raise IndexError("u(level, i, ...) outside the reference mesh")
        return float(self.array()[e])

    def __del__(self):
        if getattr(self, "h", None) and getattr(self, "_owner", False):
            try:
                lib().sg_field_destroy(self.h)
            except Exception:
                pass
            self.h = None

    def array(self):
        """u.array(): values in samurai's reference numbering (host copy)"""
        n = self.mesh.nb_cells("reference")
        out = np.empty(n, np.float64)
        _check(lib().sg_field_download(self.h, _ptr(out), n), "sg_field_download")
        return out

    def set_array(self, values):
        values = np.ascontiguousarray(values, np.float64)
        _check(lib().sg_field_upload(self.h, _ptr(values), len(values)), "sg_field_upload")

    def upload_device(self, ptr, n):
        _check(lib().sg_field_upload_device(self.h, ctypes.c_void_p(ptr), n), "sg_field_upload_device")

    def download_device(self, ptr, n):
        _check(lib().sg_field_download_device(self.h, ctypes.c_void_p(ptr), n), "sg_field_download_device")

    def set_cells(self, values):
        """u[cell] = values for every leaf cell, in for_each_cell order"""
        values = np.ascontiguousarray(values, np.float64)
        _check(lib().sg_field_set_cells(self.h, _ptr(values), len(values)), "sg_field_set_cells")

    def cell_values(self):
        n = self.mesh.nb_cells("cells")
        out = np.empty(n, np.float64)
        _check(lib().sg_field_get_cells(self.h, _ptr(out), n), "sg_field_get_cells")
        return out

    def assign_upwind(self, u, a, dt, scheme=UPWIND_OP):
        """self = u - dt * upwind(a, u) on mesh[cells]"""
        a = np.ascontiguousarray(a, np.float64)
        _check(lib().sg_upwind(u.h, self.h, _ptr(a), dt, scheme), "sg_upwind")

    def detail(self):
        n = self.mesh.nb_cells("reference")
        out = np.empty(n, np.float64)
        _check(lib().sg_detail_download(self.h, _ptr(out), n), "sg_detail_download")
        return out

    def tag(self):
        n = self.mesh.nb_cells("reference")
        out = np.empty(n, np.uint8)
        _check(lib().sg_tag_download(self.h, _ptr(out), n), "sg_tag_download")
        return out


def device_fp64_rate():
    """Measured FP64 rate of the current device (GFLOP/s, unfused add/mul)."""
    v = ctypes.c_double()
    _check(lib().sg_device_fp64_rate(ctypes.byref(v)), "sg_device_fp64_rate")
    return v.value


def make_scalar_field(name, mesh, init=None):
    """make_scalar_field<double>(name, mesh[, init_value | f]) (field/scalar_field.hpp:173-216): init a
    value for every cell, or a function of the cell centre (an array of shape (n, dim)) for the leaves"""
    u = ScalarField(name, mesh)
    if init is None:
        return u
    if callable(init):
        u.fill(0.0)
        lv, co, _ = mesh.cells()
        length = 1.0 / np.left_shift(1, lv.astype(np.int64)).astype(np.float64)
        u.set_cells(np.asarray(init(length[:, None] * (co.astype(np.float64) + 0.5)), np.float64))
    else:
        u.fill(float(init))
    return u


class Interval:
    """Interval<int, long long> (interval.hpp:51-254): [start, end), index + x = storage index"""

    __slots__ = ("start", "end", "index", "step")

    def __init__(self, start, end, index):
        self.start, self.end, self.index, self.step = int(start), int(end), int(index), 1

    def size(self):
        return self.end - self.start


def for_each_interval(mesh, f):
    """for_each_interval(mesh, f(level, i, index)) (algorithm.hpp:75-123) on the leaf cells: levels
    ascending, rows with z outer and y inner; index holds the dim-1 other coordinates"""
    for l in range(mesh.min_level(), mesh.max_level() + 1):
        for r in mesh.intervals("cells", l, with_index=True):
            f(l, Interval(r[0], r[1], r[mesh.dim + 1]), tuple(int(t) for t in r[2:mesh.dim + 1]))


class VectorField:
    """samurai::VectorField<MRMesh, double, n_comp> (field/vector_field.hpp:134-216).

    Device storage: one scalar component field per component (component-major
    slabs); host arrays keep samurai's layout, the n_comp values of a cell side
    by side (storage shape {size, n_comp}).  Every call that takes fields
    accepts a vector field and acts on its components in order, which is
    samurai's semantics: make_MRAdapt(v) tests the n_comp details together
    (mr/criteria.hpp:45-107), ghosts and upwind act component by component."""

    def __init__(self, name, mesh, n_comp):
        self.name = name
        self.mesh = mesh
        self.n_comp = int(n_comp)
        h = ctypes.c_void_p()
        _check(lib().sg_vector_field_create(mesh.h, name.encode(), self.n_comp, ctypes.byref(h)), "sg_vector_field_create")
        self.h = h
        self._comps = []
        for c in range(self.n_comp):
            ch = ctypes.c_void_p()
            _check(lib().sg_vector_field_component(h, c, ctypes.byref(ch)), "sg_vector_field_component")
            self._comps.append(ScalarField("%s_%d" % (name, c), mesh, _handle=ch))

    def __del__(self):
        if getattr(self, "h", None):
            try:
                lib().sg_vector_field_destroy(self.h)
            except Exception:
                pass
            self.h = None

    def components(self):
        return list(self._comps)

    def component(self, c):
        return self._comps[c]

    def array(self):
        """v.array(): shape (nb_reference, n_comp), samurai's reference numbering"""
        n = self.mesh.nb_cells("reference")
        out = np.empty((n, self.n_comp), np.float64)
        _check(lib().sg_vector_field_download(self.h, _ptr(out), out.size), "sg_vector_field_download")
        return out

    def set_array(self, values):
        values = np.ascontiguousarray(values, np.float64)
        _check(lib().sg_vector_field_upload(self.h, _ptr(values), values.size), "sg_vector_field_upload")

    def set_cells(self, values):
        """v[cell] = values[k] (n_comp values) for every leaf cell, in for_each_cell order"""
        values = np.ascontiguousarray(values, np.float64)
        _check(lib().sg_vector_field_set_cells(self.h, _ptr(values), values.size), "sg_vector_field_set_cells")

    def cell_values(self):
        n = self.mesh.nb_cells("cells")
        out = np.empty((n, self.n_comp), np.float64)
        _check(lib().sg_vector_field_get_cells(self.h, _ptr(out), out.size), "sg_vector_field_get_cells")
        return out

    def assign_upwind(self, u, a, dt, scheme=UPWIND_OP):
        """self = u - dt * upwind(a, u) on mesh[cells], component by component"""
        a = np.ascontiguousarray(a, np.float64)
        _check(lib().sg_vector_upwind(u.h, self.h, _ptr(a), dt, scheme), "sg_vector_upwind")


def make_vector_field(name, mesh, n_comp):
    """samurai::make_vector_field<double, n_comp>(name, mesh) (field/vector_field.hpp:232-237)"""
    return VectorField(name, mesh, n_comp)


def _components(fields):
    out = []
    for f in fields:
        out.extend(f.components())
    return out


make_field = make_scalar_field  # the README's make_field<double, 1>


class Dirichlet:
    """samurai::Dirichlet<order> (bc/dirichlet.hpp)"""

    def __init__(self, order=1):
        if order != 1:
            raise SamuraiGpuError("only Dirichlet<1> is implemented")
        self.order = order


def make_bc(bc, field, *values):
    """samurai::make_bc<Dirichlet<1>>(u, value) and make_bc<Dirichlet<1>>(v, v_0, .., v_{n-1})
    (bc/bc.hpp:752-800); no value means 0 for every component"""
    if not isinstance(bc, Dirichlet):
        raise SamuraiGpuError("only Dirichlet boundary conditions are implemented")
    comps = field.components()
    if not values:
        values = (0.0,) * len(comps)
    if len(values) != len(comps):
        raise SamuraiGpuError("make_bc: the number of constant values must equal the number of components")
    for f, v in zip(comps, values):
        _check(lib().sg_field_set_dirichlet(f.h, float(v)), "sg_field_set_dirichlet")
    return bc


class _FieldList:
    """the fields... of samurai's save / dump / load, in order (an sg_io_t)"""

    def __init__(self, fields):
        h = ctypes.c_void_p()
        _check(lib().sg_io_create(ctypes.byref(h)), "sg_io_create")
        self.h = h
        for f in fields:
            if isinstance(f, VectorField):
                _check(lib().sg_io_add_vector_field(h, f.h), "sg_io_add_vector_field")
            else:
                _check(lib().sg_io_add_field(h, f.h), "sg_io_add_field")

    def __del__(self):
        if getattr(self, "h", None):
            try:
                lib().sg_io_destroy(self.h)
            except Exception:
                pass
            self.h = None


def _io_args(args):
    """(path, filename, mesh, fields) from samurai's (path, filename, mesh, fields...)
    or (filename, mesh, fields...) forms"""
    if isinstance(args[1], MRMesh):
        return "", str(args[0]), args[1], args[2:]
    return str(args[0]), str(args[1]), args[2], args[3:]


def save(*args):
    """samurai::save(path, filename, mesh, fields...) (io/hdf5.hpp:1331-1350): <path>/<filename>.h5 and .xdmf"""
    path, filename, mesh, fields = _io_args(args)
    fl = _FieldList(fields)
    _check(lib().sg_save(path.encode(), filename.encode(), mesh.h, fl.h), "sg_save")


def dump(*args):
    """samurai::dump(path, filename, mesh, fields...) (io/restart.hpp:188-227): a restart file"""
    path, filename, mesh, fields = _io_args(args)
    fl = _FieldList(fields)
    _check(lib().sg_dump(path.encode(), filename.encode(), mesh.h, fl.h), "sg_dump")


def restart_levels(path, filename):
    """(dim, min_level, max_level) of a restart file"""
    d, lo, hi = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(lib().sg_restart_levels(path.encode(), filename.encode(), ctypes.byref(d), ctypes.byref(lo), ctypes.byref(hi)),
           "sg_restart_levels")
    return d.value, lo.value, hi.value


def load(*args):
    """samurai::load(path, filename, mesh, fields...) (io/restart.hpp:425-495): the mesh takes the file's leaf
    cells and the fields their leaf values (create the mesh with restart_levels' dimension and levels)"""
    path, filename, mesh, fields = _io_args(args)
    fl = _FieldList(fields)
    _check(lib().sg_load(path.encode(), filename.encode(), mesh.h, fl.h), "sg_load")


def swap(a, b):
    """std::swap(u.array(), unp1.array())"""
    if isinstance(a, VectorField) or isinstance(b, VectorField):
        _check(lib().sg_vector_field_swap(a.h, b.h), "sg_vector_field_swap")
        return
    _check(lib().sg_field_swap(a.h, b.h), "sg_field_swap")


def update_ghost_mr(*fields):
    """samurai::update_ghost_mr(u, ...) (algorithm/update_ghost_mr.hpp:261-270)"""
    fields = _components(fields)
    if len(fields) == 1:
        _check(lib().sg_update_ghost_mr(fields[0].h), "sg_update_ghost_mr")
        return
    hs = (ctypes.c_void_p * len(fields))(*[f.h.value for f in fields])
    _check(lib().sg_update_ghost_mr_fields(len(fields), hs), "sg_update_ghost_mr_fields")


class Adapt:
    """samurai::Adapt (mr/adapt.hpp:96-203): make_MRAdapt(u, v, ...) adapts the
    mesh to the details of all its fields; a call may carry other fields along:
    MRadaptation(mra_config, w, ...) or MRadaptation(eps, regularity, w, ...)."""

    def __init__(self, *fields):
        if not fields:
            raise SamuraiGpuError("make_MRAdapt needs at least one field")
        # a vector field contributes its components, in order (mr/adapt.hpp:74-95)
        self.fields = _components(fields)
        self.field = self.fields[0]
        self.last_harten = 0

    def __call__(self, cfg_or_eps, *args, relative_detail=False):
        if isinstance(cfg_or_eps, mra_config):
            eps, reg, rel = cfg_or_eps.epsilon(), cfg_or_eps.regularity(), cfg_or_eps.relative_detail()
            others = args
        else:
            eps, reg, rel = float(cfg_or_eps), float(args[0]), bool(relative_detail)
            others = args[1:]
        others = _components(others)
        n = ctypes.c_int()
        if len(self.fields) == 1 and not others:
            _check(lib().sg_adapt_ex(self.field.h, eps, reg, 1 if rel else 0, ctypes.byref(n)), "sg_adapt")
        else:
            fs = (ctypes.c_void_p * len(self.fields))(*[f.h.value for f in self.fields])
            os_ = (ctypes.c_void_p * max(1, len(others)))(*[f.h.value for f in others])
            _check(lib().sg_adapt_fields(len(self.fields), fs, len(others), os_, eps, reg, 1 if rel else 0, ctypes.byref(n)),
                   "sg_adapt_fields")
        self.last_harten = n.value
        return n.value

    def harten(self, ite, eps, reg, relative_detail=False):
        if len(self.fields) != 1:
            raise SamuraiGpuError("single Harten passes are exposed for one field")
        conv = ctypes.c_int()
        _check(lib().sg_harten_ex(self.field.h, ite, eps, reg, 1 if relative_detail else 0, ctypes.byref(conv)), "sg_harten")
        return bool(conv.value)


def make_MRAdapt(*fields):
    return Adapt(*fields)


class AdvectionSim:
    """One MR advection problem on the unit box with samurai's time-step
    structure (adapt, update_ghost_mr, upwind, swap), used by the tests and
    the benchmark; mirrors the oracle's driver interface."""

    def __init__(self, dim, min_level, max_level, max_stencil_radius=1, prediction_radius=1, graduation_width=1, dirichlet=0.0,
                 periodic=None):
        self.dim = dim
        self.mesh = MRMesh(dim, min_level, max_level, max_stencil_radius, prediction_radius, graduation_width, periodic=periodic)
        self.u = make_scalar_field("u", self.mesh)
        self.unp1 = make_scalar_field("unp1", self.mesh)
        make_bc(Dirichlet(1), self.u, dirichlet)
        self.adaptation = make_MRAdapt(self.u)

    def cells(self):
        return self.mesh.cells()

    def nb_cells(self):
        return self.mesh.nb_cells("cells")

    def nb_ref(self):
        return self.mesh.nb_cells("reference")

    def set_cell_values(self, values):
        self.u.set_cells(values)

    def cell_values(self):
        return self.u.cell_values()

    def field(self):
        return self.u.array()

    def set_field(self, values):
        self.u.set_array(values)

    def adapt(self, eps, regularity, relative_detail=False):
        return self.adaptation(eps, regularity, relative_detail=relative_detail)

    def harten(self, ite, eps, regularity):
        return self.adaptation.harten(ite, eps, regularity)

    def update_ghost(self):
        update_ghost_mr(self.u)

    def upwind(self, a, dt, scheme=UPWIND_OP):
        self.unp1.assign_upwind(self.u, a, dt, scheme)
        swap(self.u, self.unp1)

    def step(self, eps, regularity, a, dt, scheme=UPWIND_OP):
        """adapt, update_ghost, upwind and swap as one call (sg_step); returns the Harten passes"""
        av = np.zeros(3, np.float64)
        av[: self.dim] = np.asarray(a, np.float64)[: self.dim]
        n = ctypes.c_int()
        _check(lib().sg_step(self.u.h, self.unp1.h, float(eps), float(regularity), _ptr(av), float(dt), int(scheme), ctypes.byref(n)), "sg_step")
        return n.value

    def autotune(self, eps, regularity, a, dt, steps=10, scheme=UPWIND_OP):
        """sg_autotune: (step ms with the starting launch shape, with the chosen one, the chosen shape)"""
        av = np.zeros(3, np.float64)
        av[: self.dim] = np.asarray(a, np.float64)[: self.dim]
        d0, d1 = ctypes.c_double(), ctypes.c_double()
        _check(lib().sg_autotune(self.u.h, self.unp1.h, float(eps), float(regularity), _ptr(av), float(dt), int(scheme), int(steps),
                                 ctypes.byref(d0), ctypes.byref(d1)), "sg_autotune")
        return d0.value, d1.value, self.mesh.launch_shape()

    def intervals(self, mesh_id, level):
        return self.mesh.intervals(mesh_id, level)

    def detail(self):
        return self.u.detail()

    def tag(self):
        return self.u.tag()

    def set_cells(self, level, coords):
        self.mesh.set_cells(level, coords)


# ---------------------------------------------------------------- batched mode
class Batch:
    """Independent advection problems advanced together (the sg_batch_* calls).

    ``sims`` are AdvectionSim objects, one mesh each; ``eps``, ``regularity``,
    ``dt`` hold one value per instance and ``a`` one velocity per instance.
    Each call does, for every instance, what the serial calls on that
    instance do, with the instances running side by side on the GPU."""

    def __init__(self, sims, n_threads=8):
        self.sims = list(sims)
        n = len(self.sims)
        self._u = (ctypes.c_void_p * n)(*[s.u.h.value for s in self.sims])
        self._unp1 = (ctypes.c_void_p * n)(*[s.unp1.h.value for s in self.sims])
        h = ctypes.c_void_p()
        _check(lib().sg_batch_create(n, self._u, self._unp1, int(n_threads), ctypes.byref(h)), "sg_batch_create")
        self._h = h
        self.n_harten = np.zeros(n, dtype=np.int32)

    def __len__(self):
        return len(self.sims)

    def _params(self, values):
        v = np.ascontiguousarray(np.broadcast_to(np.asarray(values, dtype=np.float64), (len(self.sims),)))
        return v

    def _velocities(self, a):
        """one velocity for all instances, or one per instance (rows of any length <= 3)"""
        n = len(self.sims)
        rows = [a] * n if np.ndim(a[0]) == 0 else list(a)
        if len(rows) != n:
            raise SamuraiGpuError("need one velocity per instance")
        out = np.zeros((n, 3), dtype=np.float64)
        for k, r in enumerate(rows):
            out[k, : len(r)] = np.asarray(r, dtype=np.float64)
        return out

    def adapt(self, eps, regularity):
        e, r = self._params(eps), self._params(regularity)
        _check(lib().sg_batch_adapt(self._h, _ptr(e), _ptr(r), _ptr(self.n_harten)), "sg_batch_adapt")
        return self.n_harten.copy()

    def update_ghost(self):
        _check(lib().sg_batch_update_ghost_mr(self._h), "sg_batch_update_ghost_mr")

    def upwind(self, a, dt, scheme=UPWIND_OP):
        av, dv = self._velocities(a), self._params(dt)
        _check(lib().sg_batch_upwind(self._h, _ptr(av), _ptr(dv), int(scheme)), "sg_batch_upwind")
        _check(lib().sg_batch_swap(self._h), "sg_batch_swap")

    def step(self, eps, regularity, a, dt, scheme=UPWIND_OP):
        e, r, av, dv = self._params(eps), self._params(regularity), self._velocities(a), self._params(dt)
        _check(lib().sg_batch_step(self._h, _ptr(e), _ptr(r), _ptr(av), _ptr(dv), int(scheme), _ptr(self.n_harten)), "sg_batch_step")
        return self.n_harten

    def synchronize(self):
        _check(lib().sg_batch_synchronize(self._h), "sg_batch_synchronize")

    def autotune(self, eps, regularity, a, dt, steps=3, scheme=UPWIND_OP):
        """sg_batch_autotune: (batched step ms with the starting shape, with the chosen one, the chosen shape)"""
        e, r, av, dv = self._params(eps), self._params(regularity), self._velocities(a), self._params(dt)
        d0, d1 = ctypes.c_double(), ctypes.c_double()
        _check(lib().sg_batch_autotune(self._h, _ptr(e), _ptr(r), _ptr(av), _ptr(dv), int(scheme), int(steps), ctypes.byref(d0),
                                       ctypes.byref(d1)), "sg_batch_autotune")
        return d0.value, d1.value, self.launch_shape()

    def launch_shape(self):
        """{fuse_words, block} shared by the batch's instances (block 0: each instance's own)"""
        fw, bl = ctypes.c_longlong(), ctypes.c_int()
        _check(lib().sg_batch_launch_shape(self._h, ctypes.byref(fw), ctypes.byref(bl)), "sg_batch_launch_shape")
        return {"fuse_words": fw.value, "block": bl.value}

    def close(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            lib().sg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- adjoint
class Adjoint:
    """Discrete adjoint of the time loop (the sg_adjoint_* calls).

    Created from a field: its current leaf cells are the initial mesh.
    record() runs the loop with adaptation from leaf values u0 and records
    the mesh sequence; replay() reruns the recorded steps on the recorded
    meshes (the frozen-mesh map); backward() gives dJ/du0 and dJ/da at the
    last forward from dJ/duT.  Leaf values are in for_each_cell order."""

    def __init__(self, u, checkpoint_every=16):
        self.dim = u.mesh.dim
        h = ctypes.c_void_p()
        _check(lib().sg_adjoint_create(u.h, int(checkpoint_every), ctypes.byref(h)), "sg_adjoint_create")
        self._h = h

    def counts(self):
        n0, nT, ns = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
        _check(lib().sg_adjoint_counts(self._h, ctypes.byref(n0), ctypes.byref(nT), ctypes.byref(ns)), "sg_adjoint_counts")
        return n0.value, nT.value, ns.value

    def cells(self, which):
        """(level, coords) of the initial ("initial") or final ("final") mesh"""
        w = {"initial": 0, "final": 1}[which]
        n0, nT, _ = self.counts()
        n = n0 if w == 0 else nT
        lev = np.empty(n, np.int32)
        co = np.empty((n, self.dim), np.int32)
        _check(lib().sg_adjoint_cells(self._h, w, _ptr(lev), _ptr(co), n), "sg_adjoint_cells")
        return lev, co

    def _vel(self, a):
        av = np.zeros(3, np.float64)
        av[: self.dim] = np.asarray(a, np.float64)[: self.dim]
        return av

    def record(self, u0, n_steps, eps, regularity, a, dt, scheme=UPWIND_OP):
        u0 = np.ascontiguousarray(u0, np.float64)
        self.record_ptr(_ptr(u0), n_steps, eps, regularity, a, dt, scheme)
        return self.final()

    def record_ptr(self, u0_ptr, n_steps, eps, regularity, a, dt, scheme=UPWIND_OP):
        """record() from a pointer to the n0 initial leaf values: host memory or
        device memory of the mesh's GPU; returns the final leaf count"""
        nT = ctypes.c_longlong()
        av = self._vel(a)
        src = ctypes.c_void_p(u0_ptr) if isinstance(u0_ptr, int) else u0_ptr
        _check(lib().sg_adjoint_record(self._h, src, int(n_steps), float(eps), float(regularity), _ptr(av), float(dt), int(scheme),
                                       ctypes.byref(nT)), "sg_adjoint_record")
        return nT.value

    def final_ptr(self, uT_ptr, nT):
        """the final leaf values into host or device memory at uT_ptr"""
        _check(lib().sg_adjoint_final(self._h, ctypes.c_void_p(uT_ptr), int(nT)), "sg_adjoint_final")

    def backward_ptr(self, gT_ptr, g0_ptr):
        """backward() between host or device buffers: gT_ptr holds nT values,
        g0_ptr receives n0; returns dJ/da"""
        ga = np.zeros(3, np.float64)
        _check(lib().sg_adjoint_backward(self._h, ctypes.c_void_p(gT_ptr), ctypes.c_void_p(g0_ptr), _ptr(ga)), "sg_adjoint_backward")
        return ga[: self.dim].copy()

    def final(self):
        _, nT, _ = self.counts()
        out = np.empty(nT, np.float64)
        _check(lib().sg_adjoint_final(self._h, _ptr(out), nT), "sg_adjoint_final")
        return out

    def replay(self, u0, a):
        u0 = np.ascontiguousarray(u0, np.float64)
        _, nT, _ = self.counts()
        out = np.empty(nT, np.float64)
        av = self._vel(a)
        _check(lib().sg_adjoint_replay(self._h, _ptr(u0), _ptr(av), _ptr(out)), "sg_adjoint_replay")
        return out

    def backward(self, gT):
        gT = np.ascontiguousarray(gT, np.float64)
        n0, _, _ = self.counts()
        g0 = np.empty(n0, np.float64)
        ga = np.zeros(3, np.float64)
        _check(lib().sg_adjoint_backward(self._h, _ptr(gT), _ptr(g0), _ptr(ga)), "sg_adjoint_backward")
        return g0, ga[: self.dim].copy()

    def close(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            lib().sg_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
