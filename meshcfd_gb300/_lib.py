"""ctypes binding of the native library (include/meshcfd_gb300.h).

The library is built in-tree by :mod:`meshcfd_gb300.build`.  Loading fails
loudly when it is missing: there is no CPU fallback for anything here.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

from .build import BUILD, LIBNAME

_lock = threading.Lock()
_native = None

c_i32, c_i64, c_dbl, c_vp = C.c_int32, C.c_int64, C.c_double, C.c_void_p
P_i64 = C.POINTER(C.c_int64)
P_dbl = C.POINTER(C.c_double)


class Status(C.Structure):
    _fields_ = [("code", c_i32), ("first_cell", c_i32), ("first_face", c_i32), ("first_patch", c_i32)]


class Config(C.Structure):
    _fields_ = [
        ("flux", c_i32),
        ("reconstruction", c_i32),
        ("limiter", c_i32),
        ("mode", c_i32),
        ("gamma", c_dbl),
        ("acceleration_x", c_dbl),
        ("acceleration_y", c_dbl),
        ("cfl", c_dbl),
        ("gas_constant", c_dbl),
        ("viscosity_model", c_i32),
        ("reserved_i", c_i32),
        ("dynamic_viscosity", c_dbl),
        ("sutherland_reference_viscosity", c_dbl),
        ("sutherland_reference_temperature", c_dbl),
        ("sutherland_temperature", c_dbl),
        ("prandtl_number", c_dbl),
        ("venkat_k", c_dbl),
        ("reserved", c_dbl),
    ]


class GeomDesc(C.Structure):
    _fields_ = [
        ("n_cells", c_i64), ("n_faces", c_i64),
        ("areas", P_dbl), ("face_normals", P_dbl), ("face_lengths", P_dbl),
        ("owners", P_i64), ("neighbours", P_i64),
        ("n_interior", c_i64), ("interior_faces", P_i64),
        ("n_periodic", c_i64), ("periodic_faces_a", P_i64), ("periodic_faces_b", P_i64),
        ("n_wall", c_i64), ("wall_faces", P_i64), ("wall_velocities", P_dbl),
        ("n_velocity_inlet", c_i64), ("velocity_inlet_faces", P_i64), ("velocity_inlet_states", P_dbl),
        ("n_pressure_outlet", c_i64), ("pressure_outlet_faces", P_i64), ("pressure_outlet_pressures", P_dbl),
        ("n_far_field", c_i64), ("far_field_faces", P_i64), ("far_field_states", P_dbl),
        ("n_gradient", c_i64), ("gradient_sources", P_i64), ("gradient_neighbours", P_i64),
        ("gradient_coefficients_x", P_dbl), ("gradient_coefficients_y", P_dbl),
        ("n_limiter", c_i64), ("limiter_cells", P_i64), ("limiter_dx", P_dbl), ("limiter_dy", P_dbl),
        ("n_parabolic", c_i64), ("parabolic_sources", P_i64), ("parabolic_neighbours", P_i64),
        ("parabolic_dx", P_dbl), ("parabolic_dy", P_dbl),
        ("n_bc_patches", c_i64), ("bc_kind", C.POINTER(C.c_int32)), ("bc_values", P_dbl), ("bc_offsets", P_i64),
        ("bc_faces", P_i64), ("bc_direction_normal", P_dbl),
        ("gradient_dx", P_dbl), ("gradient_dy", P_dbl),
        ("n_diffusive", c_i64), ("diffusive_faces", P_i64), ("diffusive_kind", C.POINTER(C.c_int32)),
        ("diffusive_thermal", C.POINTER(C.c_int32)), ("diffusive_value", P_dbl),
        ("diffusive_inlet", C.POINTER(C.c_int32)), ("diffusive_normal_distance", P_dbl),
        ("diffusive_ghost_offset", P_dbl), ("diffusive_offset", P_dbl),
        ("interior_distance", P_dbl), ("periodic_distance", P_dbl),
    ]


class GeomInfo(C.Structure):
    _fields_ = [
        ("n_cells", c_i64), ("n_faces", c_i64), ("n_interior", c_i64), ("n_periodic", c_i64),
        ("n_boundary_flux", c_i64), ("n_flux_faces", c_i64), ("n_gradient", c_i64),
        ("n_limiter", c_i64), ("device_bytes", c_i64),
    ]


ABI_VERSION = 6  # MCFD_ABI_VERSION of include/meshcfd_gb300.h

# name -> (restype, argtypes); every symbol include/meshcfd_gb300.h declares.
SIGNATURES = {
    "mcfd_abi_version": (c_i32, []),
    "mcfd_error_string": (C.c_char_p, [c_i32]),
    "mcfd_geom_create": (c_i32, [C.POINTER(GeomDesc), C.POINTER(c_vp)]),
    "mcfd_geom_destroy": (c_i32, [c_vp]),
    "mcfd_geom_get_info": (c_i32, [c_vp, C.POINTER(GeomInfo)]),
    "mcfd_primitive": (c_i32, [c_vp, C.POINTER(Config), c_vp, c_vp, c_vp]),
    "mcfd_residual": (c_i32, [c_vp, C.POINTER(Config), c_vp, c_vp, c_vp]),
    "mcfd_time_steps": (c_i32, [c_vp, C.POINTER(Config), c_vp, c_vp, c_vp, c_dbl, c_vp]),
    "mcfd_explicit_step": (c_i32, [c_vp, C.POINTER(Config), c_i32, c_vp, c_vp, c_i32, c_vp]),
    "mcfd_explicit_step_next": (c_i32, [c_vp, C.POINTER(Config), c_i32, c_vp, c_vp, c_i32, c_i32, c_vp, c_vp, c_dbl, c_vp,
                                        c_vp]),
    "mcfd_geom_primitive": (c_vp, [c_vp]),
    "mcfd_geom_stage_state": (c_vp, [c_vp, C.c_int32]),
    "mcfd_reconstruction": (c_i32, [c_vp, C.POINTER(Config), c_vp, c_vp, c_vp, c_vp, c_vp]),
    "mcfd_explicit_step_record": (c_i32, [c_vp, C.POINTER(Config), c_i32, c_vp, c_vp, c_i32, c_vp, c_vp, c_i32,
                                          c_vp]),
    "mcfd_vjp_at": (c_i32, [c_vp, C.POINTER(Config), c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "mcfd_autotune": (c_i32, [c_vp, C.POINTER(Config), c_vp, C.POINTER(c_i32), c_vp]),
    "mcfd_set_launch_shapes": (c_i32, [c_vp, C.POINTER(c_i32)]),
    "mcfd_residual_sumsq": (c_i32, [c_vp, c_vp, c_vp, c_vp]),
    "mcfd_status_fetch": (c_i32, [c_vp, c_vp, C.POINTER(Status)]),
    "mcfd_status_fetch_next": (c_i32, [c_vp, c_vp, C.POINTER(Status)]),
    "mcfd_implicit_prepare": (c_i32, [c_vp, C.POINTER(Config), c_vp, c_vp, c_i32, P_dbl, c_vp]),
    "mcfd_implicit_matvec": (c_i32, [c_vp, c_vp, c_vp, c_vp]),
    "mcfd_implicit_set_jacobian": (c_i32, [c_vp, c_i32]),
    "mcfd_set_fused_stage": (c_i32, [c_vp, c_i32]),
    "mcfd_fused_stage_blocks": (c_i32, [c_vp]),
    "mcfd_implicit_set_sweep": (c_i32, [c_vp, c_i32, c_i32]),
    "mcfd_implicit_set_chunk": (c_i32, [c_vp, c_i32]),
    "mcfd_jvp": (c_i32, [c_vp, C.POINTER(Config), c_vp, c_vp, c_vp, c_vp]),
    "mcfd_vjp": (c_i32, [c_vp, C.POINTER(Config), c_vp, c_vp, c_vp, c_vp, c_vp]),
    "mcfd_wall_force": (c_i32, [c_vp, C.POINTER(Config), c_vp, c_dbl, c_dbl, P_dbl, c_vp, c_vp]),
    "mcfd_lusgs_apply": (c_i32, [c_vp, c_vp, c_vp, c_vp]),
    "mcfd_gmres": (c_i32, [c_vp, c_vp, c_vp, c_dbl, c_i32, c_i32, C.POINTER(c_i32), c_vp]),
    "mcfd_implicit_equation": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, P_dbl, c_vp, P_dbl, c_vp]),
    "mcfd_implicit_scale_maxima": (c_i32, [c_vp, C.POINTER(Config), c_vp, P_dbl, c_vp]),
    "mcfd_implicit_candidate": (c_i32, [c_vp, c_vp, c_vp, c_dbl, P_dbl, c_vp, c_vp]),
    "mcfd_profile_enable": (c_i32, [c_vp, c_i32]),
    "mcfd_profile_read": (c_i32, [c_vp, P_dbl, P_i64]),
    "mcfd_launch_count": (c_i64, []),
    "mcfd_batch_time_steps": (c_i32, [c_vp, C.POINTER(Config), c_vp, c_vp, c_i32, c_vp, c_vp, c_vp]),
    "mcfd_residual_sumsq_noalloc": (c_i32, [c_vp, c_i64, c_vp, c_vp]),
    "mcfd_ieee_div_sqrt": (c_i32, [c_vp, c_vp, c_i64, c_vp, c_vp, c_vp]),
    "mcfd_ieee_mul": (c_i32, [c_vp, c_vp, c_i64, c_vp, c_vp]),
    "mcfd_ieee_div_fma": (c_i32, [c_vp, c_vp, c_i64, c_vp, c_vp]),
    "mcfd_host_cell_geometry": (c_i32, [c_i64, P_i64, P_i64, P_dbl, P_dbl, P_dbl, P_i64]),
    "mcfd_host_face_geometry": (c_i32, [c_i64, P_i64, P_dbl, P_dbl, P_i64, P_dbl, P_dbl, P_dbl, P_i64]),
    "mcfd_device_cell_geometry": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "mcfd_device_face_geometry": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "mcfd_device_gradient_coefficients": (c_i32, [c_i64, c_i64, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                                  c_vp, c_vp, c_vp, c_vp, c_vp]),
    "mcfd_device_limiter_offsets": (c_i32, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "mcfd_host_parabolic_stencil": (c_i32, [c_i64, c_i64, P_i64, P_i64, P_dbl, P_dbl, c_dbl, c_i64, P_i64, P_i64,
                                            P_dbl, P_dbl, P_i64]),
}


class NativeError(RuntimeError):
    pass


def _ptr(a: np.ndarray, kind):
    return a.ctypes.data_as(kind) if a is not None and a.size else None


class Native:
    """Thin wrapper: raw ctypes functions plus NumPy-friendly host helpers."""

    def __init__(self, path: Path):
        self.path = path
        self.lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(self.lib, name)
            fn.restype = res
            fn.argtypes = args
            setattr(self, name, fn)
        if self.mcfd_abi_version() != ABI_VERSION:
            raise NativeError(f"{path}: ABI version {self.mcfd_abi_version()}, expected {ABI_VERSION} (rebuild)")

    def check(self, rc: int, what: str) -> None:
        if rc != 0:
            raise NativeError(f"{what}: {self.mcfd_error_string(rc).decode()} (code {rc})")

    def cell_geometry(self, offsets, nodes, points):
        from .errors import SolverError

        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        nodes = np.ascontiguousarray(nodes, dtype=np.int64)
        points = np.ascontiguousarray(points, dtype=np.float64)
        n = len(offsets) - 1
        centers = np.empty((n, 2))
        areas = np.empty(n)
        bad = C.c_int64(-1)
        rc = self.mcfd_host_cell_geometry(n, _ptr(offsets, P_i64), _ptr(nodes, P_i64), _ptr(points, P_dbl),
                                          _ptr(centers, P_dbl), _ptr(areas, P_dbl), C.byref(bad))
        if rc == 4:
            raise SolverError(f"Cell {bad.value} has zero or invalid area.")
        self.check(rc, "cell geometry")
        return centers, areas

    def face_geometry(self, faces, points, centers, owners):
        from .errors import SolverError

        faces = np.ascontiguousarray(faces, dtype=np.int64)
        owners = np.ascontiguousarray(owners, dtype=np.int64)
        n = len(faces)
        fc = np.empty((n, 2))
        normals = np.empty((n, 2))
        lengths = np.empty(n)
        bad = C.c_int64(-1)
        rc = self.mcfd_host_face_geometry(n, _ptr(faces, P_i64), _ptr(np.ascontiguousarray(points), P_dbl),
                                          _ptr(np.ascontiguousarray(centers), P_dbl), _ptr(owners, P_i64),
                                          _ptr(fc, P_dbl), _ptr(normals, P_dbl), _ptr(lengths, P_dbl), C.byref(bad))
        if rc == 4:
            raise SolverError(f"Face {bad.value} has zero or invalid length.")
        self.check(rc, "face geometry")
        return fc, normals, lengths


    def parabolic_stencil(self, cell_count, sources, neighbours, dx, dy, domain_scale):
        """The two-ring stencil (solver.py:2241-2291) by the compiled search
        (mcfd_host_parabolic_stencil); the same entries as
        ``geometry.parabolic_stencil``."""
        sources = np.ascontiguousarray(sources, dtype=np.int64)
        neighbours = np.ascontiguousarray(neighbours, dtype=np.int64)
        dx = np.ascontiguousarray(dx, dtype=np.float64)
        dy = np.ascontiguousarray(dy, dtype=np.float64)
        degree = np.bincount(sources, minlength=cell_count) if len(sources) else np.zeros(cell_count, np.int64)
        capacity = int(len(sources) + degree[neighbours].sum()) if len(sources) else 0
        out_s = np.empty(max(capacity, 1), dtype=np.int64)
        out_n = np.empty_like(out_s)
        out_x = np.empty(max(capacity, 1))
        out_y = np.empty_like(out_x)
        count = C.c_int64(0)
        rc = self.mcfd_host_parabolic_stencil(int(cell_count), len(sources), _ptr(sources, P_i64),
                                              _ptr(neighbours, P_i64), _ptr(dx, P_dbl), _ptr(dy, P_dbl),
                                              float(domain_scale), capacity, _ptr(out_s, P_i64), _ptr(out_n, P_i64),
                                              _ptr(out_x, P_dbl), _ptr(out_y, P_dbl), C.byref(count))
        self.check(rc, "parabolic stencil")
        n = count.value
        return out_s[:n].copy(), out_n[:n].copy(), out_x[:n].copy(), out_y[:n].copy()


def library_path() -> Path:
    return BUILD / LIBNAME


def native() -> Native:
    """Load (building first if the sources are newer) the native library."""
    global _native
    with _lock:
        if _native is None:
            from .build import build

            path = build()
            if not path.exists():
                raise NativeError(f"native library missing: {path}")
            _native = Native(path)
        return _native
