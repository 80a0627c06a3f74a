"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product package never does.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        vp, i, d, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [i, i, i, i, i, i, d]
        L.oracle_create_periodic.restype = vp
        L.oracle_create_periodic.argtypes = [i, i, i, i, i, i, d, i]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_nb_cells.restype = ll
        L.oracle_nb_cells.argtypes = [vp]
        L.oracle_nb_ref.restype = ll
        L.oracle_nb_ref.argtypes = [vp]
        L.oracle_get_cells.argtypes = [vp, vp, vp, vp]
        L.oracle_get_field.argtypes = [vp, vp]
        L.oracle_set_field.argtypes = [vp, vp]
        L.oracle_get_detail.argtypes = [vp, vp]
        L.oracle_get_tag.argtypes = [vp, vp]
        L.oracle_adapt.restype = i
        L.oracle_adapt.argtypes = [vp, d, d]
        L.oracle_adapt_rel.restype = i
        L.oracle_adapt_rel.argtypes = [vp, d, d, i]
        L.oracle_add_field.restype = i
        L.oracle_add_field.argtypes = [vp, d]
        L.oracle_get_field_k.argtypes = [vp, i, vp]
        L.oracle_set_field_k.argtypes = [vp, i, vp]
        L.oracle_update_ghost_k.restype = i
        L.oracle_update_ghost_k.argtypes = [vp, i]
        L.oracle_adapt_fields.restype = i
        L.oracle_adapt_fields.argtypes = [vp, d, d, i, i, i]
        L.oracle_harten.restype = i
        L.oracle_harten.argtypes = [vp, i, d, d]
        L.oracle_update_ghost.restype = i
        L.oracle_update_ghost.argtypes = [vp]
        L.oracle_upwind.restype = i
        L.oracle_upwind.argtypes = [vp, vp, d, i]
        L.oracle_upwind_k.restype = i
        L.oracle_upwind_k.argtypes = [vp, i, vp, d, i]
        L.oracle_count_intervals.restype = ll
        L.oracle_count_intervals.argtypes = [vp, i, i]
        L.oracle_get_intervals.argtypes = [vp, i, i, vp]
        L.oracle_set_cells.restype = i
        L.oracle_set_cells.argtypes = [vp, ll, vp, vp]
        L.oracle_set_refine_boundary.argtypes = [vp, i]
        L.oracle_transfer_cells.restype = i
        L.oracle_transfer_cells.argtypes = [vp, ll, vp, vp]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


MESH_IDS = {"cells": 0, "cells_and_ghosts": 1, "proj_cells": 2, "union_cells": 3, "reference": 4}


class OracleSim:
    """One MR advection problem on the unit box, driven step by step."""

    def __init__(self, dim, min_level, max_level, max_stencil_radius=1, prediction_radius=1, graduation_width=1, dirichlet=0.0,
                 periodic=(False, False, False)):
        """periodic: one flag per axis (mesh_config::periodic)"""
        self.dim = dim
        self.min_level = min_level
        self.max_level = max_level
        mask = sum(1 << d for d, p in enumerate(periodic) if p)
        self.h = lib().oracle_create_periodic(dim, min_level, max_level, max_stencil_radius, prediction_radius, graduation_width, dirichlet,
                                              mask)
        if not self.h:
            raise RuntimeError("oracle_create failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    def nb_cells(self):
        return lib().oracle_nb_cells(self.h)

    def nb_ref(self):
        return lib().oracle_nb_ref(self.h)

    def cells(self):
        n = self.nb_cells()
        level = np.empty(n, np.int32)
        coords = np.empty((n, self.dim), np.int32)
        index = np.empty(n, np.int64)
        lib().oracle_get_cells(self.h, _ptr(level), _ptr(coords), _ptr(index))
        return level, coords, index

    def field(self):
        out = np.empty(self.nb_ref(), np.float64)
        lib().oracle_get_field(self.h, _ptr(out))
        return out

    def set_field(self, u):
        u = np.ascontiguousarray(u, np.float64)
        assert u.shape == (self.nb_ref(),)
        lib().oracle_set_field(self.h, _ptr(u))

    def set_cell_values(self, values):
        """Set the leaf-cell values (for_each_cell order); ghosts become NaN."""
        _, _, index = self.cells()
        u = np.full(self.nb_ref(), np.nan)
        u[index] = values
        self.set_field(u)

    def cell_values(self):
        _, _, index = self.cells()
        return self.field()[index]

    def detail(self):
        out = np.empty(self.nb_ref(), np.float64)
        lib().oracle_get_detail(self.h, _ptr(out))
        return out

    def tag(self):
        out = np.empty(self.nb_ref(), np.uint8)
        lib().oracle_get_tag(self.h, _ptr(out))
        return out

    def adapt(self, eps, regularity, relative_detail=False):
        r = lib().oracle_adapt_rel(self.h, eps, regularity, 1 if relative_detail else 0)
        if r < 0:
            raise RuntimeError("oracle adapt failed")
        return r

    def harten(self, ite, eps, regularity):
        r = lib().oracle_harten(self.h, ite, eps, regularity)
        if r < 0:
            raise RuntimeError("oracle harten failed")
        return bool(r)

    def update_ghost(self):
        if lib().oracle_update_ghost(self.h) != 0:
            raise RuntimeError("oracle update_ghost failed")

    def upwind(self, a, dt, scheme=0):
        a = np.ascontiguousarray(a, np.float64)
        if lib().oracle_upwind(self.h, _ptr(a), dt, scheme) != 0:
            raise RuntimeError("oracle upwind failed")

    def intervals(self, mesh_id, level):
        mid = MESH_IDS[mesh_id] if isinstance(mesh_id, str) else mesh_id
        n = lib().oracle_count_intervals(self.h, mid, level)
        out = np.empty((n, self.dim + 1), np.int32)
        lib().oracle_get_intervals(self.h, mid, level, _ptr(out))
        return out

    def set_cells(self, level, coords):
        level = np.ascontiguousarray(level, np.int32)
        coords = np.ascontiguousarray(coords, np.int32)
        if lib().oracle_set_cells(self.h, len(level), _ptr(level), _ptr(coords)) != 0:
            raise RuntimeError("oracle set_cells failed")

    def set_refine_boundary(self, enable):
        """--refine-boundary (args::refine_boundary) for the adaptations of this problem"""
        lib().oracle_set_refine_boundary(self.h, 1 if enable else 0)

    def transfer_cells(self, level, coords):
        """the mesh becomes that of the given leaf cells; the field follows it
        through update_fields (one recorded transition of a frozen-mesh replay)"""
        level = np.ascontiguousarray(level, np.int32)
        coords = np.ascontiguousarray(coords, np.int32)
        if lib().oracle_transfer_cells(self.h, len(level), _ptr(level), _ptr(coords)) != 0:
            raise RuntimeError("oracle transfer_cells failed")

    # ---- more fields on the same mesh (field 0 is the one above)
    def add_field(self, dirichlet=0.0):
        """a new field (values undefined until set), with Dirichlet<1> value"""
        return lib().oracle_add_field(self.h, dirichlet)

    def field_k(self, k):
        out = np.empty(self.nb_ref(), np.float64)
        lib().oracle_get_field_k(self.h, k, _ptr(out))
        return out

    def set_cell_values_k(self, k, values):
        _, _, index = self.cells()
        u = np.full(self.nb_ref(), np.nan)
        u[index] = values
        lib().oracle_set_field_k(self.h, k, _ptr(np.ascontiguousarray(u)))

    def cell_values_k(self, k):
        _, _, index = self.cells()
        return self.field_k(k)[index]

    def update_ghost_k(self, k):
        if lib().oracle_update_ghost_k(self.h, k) != 0:
            raise RuntimeError("oracle update_ghost failed")

    def upwind_k(self, k, a, dt, scheme=0):
        a = np.ascontiguousarray(a, np.float64)
        if lib().oracle_upwind_k(self.h, k, _ptr(a), dt, scheme) != 0:
            raise RuntimeError("oracle upwind failed")

    def adapt_fields(self, eps, regularity, n_crit, n_other=0, relative_detail=False):
        """make_MRAdapt(f_0..f_{n_crit-1})(mra_config, others): returns the Harten passes"""
        r = lib().oracle_adapt_fields(self.h, eps, regularity, 1 if relative_detail else 0, n_crit, n_other)
        if r < 0:
            raise RuntimeError("oracle adapt failed")
        return r
