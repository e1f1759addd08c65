"""Device geometry handle and the host-side calls of the C ABI.

A :class:`DeviceGeometry` is built once per mesh from a reference
``_Geometry`` (solver.py:123-177) or from :func:`meshcfd_gb300.geometry.
build_geometry`; it owns the packed device arrays and workspace.  States are
torch float64 tensors of shape (n_cells, 4) on the handle's CUDA device.
"""

from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib
from .errors import SolverError, StatusCode, raise_for_status
from .model import (EXTENSION_LIMITER_CODES, FLUX_CODES, LIMITER_CODES, RECONSTRUCTION_CODES,
                    VENKATAKRISHNAN_K_DEFAULT)

TIME_SCHEME_CODES = {"Explicit Euler": 0, "Explicit RK2": 1, "Explicit RK3": 2, "Explicit RK4": 3}


MODES = {"exact": 0, "fast": 1, "fma": 2}


def make_config(settings, mode: str = "exact") -> _lib.Config:
    """Map ``NumericalSettings`` (model.py:95-129) to the kernel config.

    ``mode``: "exact" (reference operation order, bit-exact), "fast" (exact
    arithmetic, limiter minimum through the smallest ratio) or "fma" (shared
    reciprocals and FMA; outside the 1e-12 bar on fine meshes).  MUSCL
    parabolic reconstructs with exact arithmetic in every mode.  The limiter
    "Venkatakrishnan K" (an extension, code 4) reads K from the settings
    attribute ``venkatakrishnan_k``."""
    viscous = {"Inviscid": 0, "Constant": 1, "Sutherland": 2}
    if settings.viscosity_model not in viscous:
        raise SolverError(f"Unsupported viscosity model '{settings.viscosity_model}'.")
    if settings.turbulence_model != "None":
        raise NotImplementedError("SST turbulence is not implemented by the GPU residual path")
    try:
        flux = FLUX_CODES[settings.flux]
        recon = RECONSTRUCTION_CODES[settings.reconstruction]
        limiter = {**LIMITER_CODES, **EXTENSION_LIMITER_CODES}[settings.limiter]
    except KeyError as error:
        raise SolverError(f"Unsupported scheme {error}") from error
    cfg = _lib.Config()
    cfg.flux, cfg.reconstruction, cfg.limiter, cfg.mode = flux, recon, limiter, MODES[mode]
    cfg.gamma = float(settings.gamma)
    cfg.acceleration_x = float(settings.acceleration_x)
    cfg.acceleration_y = float(settings.acceleration_y)
    cfg.cfl = float(settings.cfl)
    cfg.gas_constant = float(settings.gas_constant)
    cfg.viscosity_model = viscous[settings.viscosity_model]
    cfg.dynamic_viscosity = float(settings.dynamic_viscosity)
    cfg.sutherland_reference_viscosity = float(settings.sutherland_reference_viscosity)
    cfg.sutherland_reference_temperature = float(settings.sutherland_reference_temperature)
    cfg.sutherland_temperature = float(settings.sutherland_temperature)
    cfg.prandtl_number = float(settings.prandtl_number)
    cfg.venkat_k = float(getattr(settings, "venkatakrishnan_k", VENKATAKRISHNAN_K_DEFAULT))
    return cfg


def primitive_to_conservative(primitive, gamma: float) -> np.ndarray:
    """Host conversion (rho, u, v, p) -> (rho, rho u, rho v, E) in the
    reference's expression order (euler.py:8-17)."""
    P = np.asarray(primitive, dtype=np.float64)
    rho, u, v, p = P.T
    E = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return np.column_stack((rho, rho * u, rho * v, E))


def _stream_ptr(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _check_state(x: torch.Tensor, n_cells: int, name: str) -> None:
    if x.dtype != torch.float64 or not x.is_cuda or x.shape != (n_cells, 4) or not x.is_contiguous():
        raise ValueError(f"{name} must be a contiguous CUDA float64 tensor of shape ({n_cells}, 4)")


def geometry_descriptor(geometry):
    """The `mcfd_geom_desc` of a host geometry (the reference `_Geometry`
    arrays, plus the boundary-patch and viscous tables when present), the
    NumPy arrays it points into (keep them alive while the descriptor is in
    use) and the boundary-patch names.  Needs no device."""
    keep = {}

    def a(name, dtype, shape=None, src=None):
        v = getattr(geometry, name) if src is None else src
        arr = np.ascontiguousarray(np.asarray(v, dtype=dtype))
        if shape is not None:
            arr = arr.reshape(shape)
        keep[name] = arr
        kind = _lib.P_i64 if dtype == np.int64 else _lib.P_dbl
        return arr.ctypes.data_as(kind) if arr.size else None, len(arr)

    d = _lib.GeomDesc()
    d.areas, n_cells = a("areas", np.float64)
    d.face_lengths, n_faces = a("face_lengths", np.float64)
    d.n_cells, d.n_faces = n_cells, n_faces
    d.face_normals, _ = a("face_normals", np.float64, (-1, 2))
    d.owners, _ = a("owners", np.int64)
    d.neighbours, _ = a("neighbours", np.int64)
    d.interior_faces, d.n_interior = a("interior_faces", np.int64)
    d.periodic_faces_a, d.n_periodic = a("periodic_faces_a", np.int64)
    d.periodic_faces_b, _ = a("periodic_faces_b", np.int64)
    d.wall_faces, d.n_wall = a("wall_faces", np.int64)
    d.wall_velocities, _ = a("wall_velocities", np.float64, (-1, 2))
    d.velocity_inlet_faces, d.n_velocity_inlet = a("velocity_inlet_faces", np.int64)
    d.velocity_inlet_states, _ = a("velocity_inlet_states", np.float64, (-1, 4))
    d.pressure_outlet_faces, d.n_pressure_outlet = a("pressure_outlet_faces", np.int64)
    d.pressure_outlet_pressures, _ = a("pressure_outlet_pressures", np.float64)
    d.far_field_faces, d.n_far_field = a("far_field_faces", np.int64)
    d.far_field_states, _ = a("far_field_states", np.float64, (-1, 4))
    d.gradient_sources, d.n_gradient = a("gradient_sources", np.int64)
    d.gradient_neighbours, _ = a("gradient_neighbours", np.int64)
    d.gradient_coefficients_x, _ = a("gradient_coefficients_x", np.float64)
    d.gradient_coefficients_y, _ = a("gradient_coefficients_y", np.float64)
    d.limiter_cells, d.n_limiter = a("limiter_cells", np.int64)
    d.limiter_dx, _ = a("limiter_dx", np.float64)
    d.limiter_dy, _ = a("limiter_dy", np.float64)
    empty_i, empty_d = np.empty(0, dtype=np.int64), np.empty(0)
    d.parabolic_sources, d.n_parabolic = a("parabolic_sources", np.int64,
                                           src=getattr(geometry, "parabolic_sources", empty_i))
    d.parabolic_neighbours, _ = a("parabolic_neighbours", np.int64,
                                  src=getattr(geometry, "parabolic_neighbours", empty_i))
    d.parabolic_dx, _ = a("parabolic_dx", np.float64, src=getattr(geometry, "parabolic_dx", empty_d))
    d.parabolic_dy, _ = a("parabolic_dy", np.float64, src=getattr(geometry, "parabolic_dy", empty_d))
    bc = boundary_patches(geometry)
    d.n_bc_patches = len(bc["names"])
    if d.n_bc_patches:
        keep["bc_kind"] = bc["kind"]
        d.bc_kind = bc["kind"].ctypes.data_as(C.POINTER(C.c_int32))
        d.bc_values, _ = a("bc_values", np.float64, src=bc["values"])
        d.bc_offsets, _ = a("bc_offsets", np.int64, src=bc["offsets"])
        d.bc_faces, _ = a("bc_faces", np.int64, src=bc["faces"])
        d.bc_direction_normal, _ = a("bc_direction_normal", np.float64, src=bc["direction_normal"])
    vt = viscous_tables(geometry, bc) \
        if hasattr(geometry, "diffusive_boundary_faces") and hasattr(geometry, "gradient_dx") else None
    if vt is not None:
        d.gradient_dx, _ = a("gradient_dx", np.float64)
        d.gradient_dy, _ = a("gradient_dy", np.float64)
        d.diffusive_faces, d.n_diffusive = a("diffusive_faces", np.int64, src=vt["faces"])
        for name in ("kind", "thermal", "inlet"):
            arr = vt[name]
            keep["diffusive_" + name] = arr
            setattr(d, "diffusive_" + name, arr.ctypes.data_as(C.POINTER(C.c_int32)) if arr.size else None)
        d.diffusive_value, _ = a("diffusive_value", np.float64, src=vt["value"])
        d.diffusive_normal_distance, _ = a("diffusive_nd", np.float64, src=vt["nd"])
        d.diffusive_ghost_offset, _ = a("diffusive_ghost", np.float64, src=vt["ghost"])
        d.diffusive_offset, _ = a("diffusive_offset", np.float64, src=vt["offset"])
        d.interior_distance, _ = a("interior_distance", np.float64, src=vt["interior_distance"])
        d.periodic_distance, _ = a("periodic_distance", np.float64, src=vt["periodic_distance"])
    return d, keep, bc["names"]


class DeviceGeometry:
    """Packed device geometry + workspace for one mesh (one CUDA device)."""

    def __init__(self, geometry, device=None):
        self.lib = _lib.native()
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else torch.device(device).index or 0)
        d, keep, self.bc_patch_names = geometry_descriptor(geometry)
        n_cells = int(d.n_cells)
        handle = C.c_void_p()
        with torch.cuda.device(self.device):
            rc = self.lib.mcfd_geom_create(C.byref(d), C.byref(handle))
        if rc == 4:
            raise SolverError("device geometry: inconsistent geometry arrays")
        self.lib.check(rc, "mcfd_geom_create")
        self.handle = handle.value
        info = _lib.GeomInfo()
        self.lib.check(self.lib.mcfd_geom_get_info(self.handle, C.byref(info)), "mcfd_geom_get_info")
        self.info = info
        self.n_cells = int(info.n_cells)
        self.n_faces = int(info.n_faces)
        self.n_interior = int(info.n_interior)
        self.n_far_field = int(d.n_far_field)
        self.areas = torch.as_tensor(keep["areas"], device=self.device)
        owners = keep["owners"]
        # owner cell of every far-field face and the wall-force weight of
        # every cell, sum over its wall / symmetry faces of n L (the adjoint's
        # per-cell time steps and per-case functionals)
        self.far_owner = torch.as_tensor(owners[keep["far_field_faces"]], device=self.device)
        wall = keep["wall_faces"]
        normals = keep["face_normals"].reshape(-1, 2)
        wn = np.zeros((n_cells, 2))
        np.add.at(wn, owners[wall], normals[wall] * keep["face_lengths"][wall, None])
        self.wall_normal_length = torch.as_tensor(wn, device=self.device)
        self._dt_min = torch.empty(1, dtype=torch.float64, device=self.device)

    # ------------------------------------------------------------- lifetime
    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.mcfd_geom_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --------------------------------------------------------------- status
    def check_status(self, solver_error=SolverError, stream=None) -> None:
        raise_for_status(self.status_code(stream), solver_error)

    def status_code(self, stream=None, *, look_ahead: bool = False) -> StatusCode:
        """The device status bits since the last fetch (an int), carrying the
        name of the lowest failing boundary patch as ``.patch``.
        ``look_ahead``: the word of the next step's time steps that
        :meth:`explicit_step_next` computes (mcfd_status_fetch_next)."""
        st = _lib.Status()
        fetch = self.lib.mcfd_status_fetch_next if look_ahead else self.lib.mcfd_status_fetch
        self.lib.check(fetch(self.handle, _stream_ptr(stream), C.byref(st)), "mcfd_status_fetch")
        code = StatusCode(st.code)
        if 0 <= st.first_patch < len(self.bc_patch_names):
            code.patch = self.bc_patch_names[st.first_patch]
        return code

    # ----------------------------------------------------------- operations
    def primitive(self, U: torch.Tensor, cfg, out: torch.Tensor | None = None) -> torch.Tensor:
        _check_state(U, self.n_cells, "U")
        P = torch.empty_like(U) if out is None else out
        self.lib.check(self.lib.mcfd_primitive(self.handle, C.byref(cfg), U.data_ptr(), P.data_ptr(), _stream_ptr()),
                       "mcfd_primitive")
        return P

    def residual(self, U: torch.Tensor, cfg, out: torch.Tensor | None = None) -> torch.Tensor:
        _check_state(U, self.n_cells, "U")
        R = torch.empty_like(U) if out is None else out
        self.lib.check(self.lib.mcfd_residual(self.handle, C.byref(cfg), U.data_ptr(), R.data_ptr(), _stream_ptr()),
                       "mcfd_residual")
        return R

    def reconstruction(self, P: torch.Tensor, cfg):
        """(gradients (C,4,2), curvature (C,4,3) or None, factors (C,4)) of
        _limited_gradients / _parabolic_reconstruction (solver.py:2294-2415)."""
        _check_state(P, self.n_cells, "P")
        grad = torch.empty(self.n_cells, 4, 2, dtype=torch.float64, device=self.device)
        fac = torch.empty(self.n_cells, 4, dtype=torch.float64, device=self.device)
        curv = torch.empty(self.n_cells, 4, 3, dtype=torch.float64, device=self.device) if cfg.reconstruction == 2 else None
        self.lib.check(self.lib.mcfd_reconstruction(self.handle, C.byref(cfg), P.data_ptr(), grad.data_ptr(),
                                                    curv.data_ptr() if curv is not None else None, fac.data_ptr(),
                                                    _stream_ptr()), "mcfd_reconstruction")
        return grad, curv, fac

    def autotune(self, U: torch.Tensor, cfg) -> dict:
        """Time the stage kernels' launch shapes on state U and keep the
        fastest for this handle (mcfd_autotune)."""
        _check_state(U, self.n_cells, "U")
        chosen = (C.c_int32 * 5)()
        self.lib.check(self.lib.mcfd_autotune(self.handle, C.byref(cfg), U.data_ptr(), chosen, _stream_ptr()),
                       "mcfd_autotune")
        return {"reconstruct_threads": chosen[0], "flux_threads": chosen[1], "flux_faces_per_thread": chosen[2],
                "gather_threads": chosen[3], "reconstruct_per_variable": chosen[4]}

    def set_fused_stage(self, on: bool) -> None:
        """Run each explicit stage as one cooperative launch (reconstruction,
        fluxes and gather separated by grid barriers) where the settings allow
        it (mcfd_set_fused_stage); results are identical either way."""
        self.lib.check(self.lib.mcfd_set_fused_stage(self.handle, 1 if on else 0), "mcfd_set_fused_stage")

    @property
    def fused_stage_blocks(self) -> int:
        """Resident blocks per SM of the last one-launch stage (0 before any)."""
        return int(self.lib.mcfd_fused_stage_blocks(self.handle))

    def primitive_buffer(self) -> torch.Tensor:
        """The handle's primitive buffer as a tensor view (valid after a
        residual / primitive / step call)."""
        ptr = self.lib.mcfd_geom_primitive(self.handle)
        return _device_view(ptr, (self.n_cells, 4), self.device)

    def time_steps(self, P: torch.Tensor, cfg, time_limit: float = math.inf, per_cell: bool = False,
                   out_min: torch.Tensor | None = None):
        _check_state(P, self.n_cells, "P")
        dt_cells = torch.empty(self.n_cells, dtype=torch.float64, device=self.device) if per_cell else None
        dt_min = self._dt_min if out_min is None else out_min
        self.lib.check(self.lib.mcfd_time_steps(self.handle, C.byref(cfg), P.data_ptr(),
                                                dt_cells.data_ptr() if dt_cells is not None else None,
                                                dt_min.data_ptr(), float(time_limit), _stream_ptr()),
                       "mcfd_time_steps")
        return dt_cells, dt_min

    def explicit_step(self, U: torch.Tensor, cfg, scheme: int, dt: torch.Tensor) -> None:
        _check_state(U, self.n_cells, "U")
        if dt.dtype != torch.float64 or not dt.is_cuda or dt.numel() not in (1, self.n_cells):
            raise ValueError("dt must be a CUDA float64 tensor with 1 or n_cells elements")
        per_cell = int(dt.numel() == self.n_cells and self.n_cells != 1)
        self.lib.check(self.lib.mcfd_explicit_step(self.handle, C.byref(cfg), int(scheme), U.data_ptr(), dt.data_ptr(),
                                                   per_cell, _stream_ptr()), "mcfd_explicit_step")

    def explicit_step_next(self, U: torch.Tensor, cfg, scheme: int, dt: torch.Tensor, *,
                           next_dt_min: torch.Tensor | None = None, next_dt_cells: torch.Tensor | None = None,
                           time_limit: float = math.inf, primitive_current: bool = False,
                           start_residual: torch.Tensor | None = None) -> None:
        """One explicit step that also leaves the next step's stable time
        steps (mcfd_explicit_step_next): per cell into ``next_dt_cells``
        and / or their minimum with ``time_limit`` into ``next_dt_min``.
        ``primitive_current``: the handle's primitive buffer holds the
        primitive of U (as the previous step left it).  The time steps'
        status bits are read by ``status_code(look_ahead=True)``.
        ``start_residual``: (C,4) float64, receives the residual of U that
        the first stage computes."""
        _check_state(U, self.n_cells, "U")
        if start_residual is not None:
            _check_state(start_residual, self.n_cells, "start_residual")
        if dt.dtype != torch.float64 or not dt.is_cuda or dt.numel() not in (1, self.n_cells):
            raise ValueError("dt must be a CUDA float64 tensor with 1 or n_cells elements")
        for name, t, n in (("next_dt_min", next_dt_min, 1), ("next_dt_cells", next_dt_cells, self.n_cells)):
            if t is not None and (t.dtype != torch.float64 or not t.is_cuda or t.numel() != n):
                raise ValueError(f"{name} must be a CUDA float64 tensor with {n} elements")
        per_cell = int(dt.numel() == self.n_cells and self.n_cells != 1)
        self.lib.check(self.lib.mcfd_explicit_step_next(
            self.handle, C.byref(cfg), int(scheme), U.data_ptr(), dt.data_ptr(), per_cell, int(primitive_current),
            next_dt_cells.data_ptr() if next_dt_cells is not None else None,
            next_dt_min.data_ptr() if next_dt_min is not None else None, float(time_limit),
            start_residual.data_ptr() if start_residual is not None else None, _stream_ptr()),
            "mcfd_explicit_step_next")

    def residual_sumsq(self, R: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        _check_state(R, self.n_cells, "R")
        sums = torch.empty(4, dtype=torch.float64, device=self.device) if out is None else out
        self.lib.check(self.lib.mcfd_residual_sumsq(self.handle, R.data_ptr(), sums.data_ptr(), _stream_ptr()),
                       "mcfd_residual_sumsq")
        return sums


BC_PRESSURE_INLET, BC_MASS_FLOW_INLET, BC_MASS_FLOW_OUTLET = 0, 1, 2


def boundary_patches(geometry) -> dict:
    """The pressure-inlet, mass-flow-inlet and mass-flow-outlet patches of a
    geometry (solver.py:81-103) as the C ABI's patch table, in the order the
    residual visits them (solver.py:2626-2698).  The per-face n . direction is
    NumPy's own ``normals @ direction`` (solver.py:4423, 4507), whose BLAS
    rounding the states depend on; the outlet's total length is NumPy's own
    ``np.sum`` (solver.py:4568)."""
    normals_all = np.asarray(geometry.face_normals, dtype=np.float64).reshape(-1, 2)
    lengths_all = np.asarray(geometry.face_lengths, dtype=np.float64)
    names, kinds, values, offsets, faces, dn = [], [], [], [0], [], []
    for kind, patches in ((BC_PRESSURE_INLET, getattr(geometry, "pressure_inlets", ())),
                          (BC_MASS_FLOW_INLET, getattr(geometry, "mass_flow_inlets", ())),
                          (BC_MASS_FLOW_OUTLET, getattr(geometry, "mass_flow_outlets", ()))):
        for b in patches:
            f = np.asarray(b.faces, dtype=np.int64)
            if kind == BC_PRESSURE_INLET:
                if not math.isclose(float(np.linalg.norm(b.direction)), 1.0):  # solver.py:4420-4423
                    raise SolverError(f"Pressure inlet '{b.patch_name}' has an invalid flow direction.")
                values.append((b.total_pressure, b.total_temperature, b.direction[0], b.direction[1]))
                dn.append(normals_all[f] @ np.asarray(b.direction, dtype=np.float64))
            elif kind == BC_MASS_FLOW_INLET:
                values.append((b.mass_flow, b.total_temperature, b.direction[0], b.direction[1]))
                dn.append(normals_all[f] @ np.asarray(b.direction, dtype=np.float64))
            else:
                values.append((b.mass_flow, float(np.sum(lengths_all[f])), 0.0, 0.0))
                dn.append(np.zeros(len(f)))
            names.append(b.patch_name)
            kinds.append(kind)
            faces.append(f)
            offsets.append(offsets[-1] + len(f))
    cat = (lambda parts, dtype: np.concatenate(parts).astype(dtype) if parts else np.empty(0, dtype=dtype))
    return {"names": names, "kind": np.asarray(kinds, dtype=np.int32),
            "values": np.asarray(values, dtype=np.float64).reshape(-1, 4),
            "offsets": np.asarray(offsets, dtype=np.int64), "faces": cat(faces, np.int64),
            "direction_normal": cat(dn, np.float64)}


DIFF_WALL_NO_SLIP, DIFF_WALL_SLIP, DIFF_SYMMETRY, DIFF_INLET, DIFF_OTHER, DIFF_WALL_UNKNOWN = range(6)


def viscous_tables(geometry, bc) -> dict:
    """The laminar viscous tables of the C ABI for a geometry: per diffusive
    boundary face (solver.py:1817-1820) its kind, wall thermal data, inlet
    state source, the normal distance and ghost offset exactly as the
    reference computes them (NumPy's own np.dot, solver.py:3651-3655), and
    the time step's face distances (solver.py:4266-4299)."""
    owners = np.asarray(geometry.owners)
    neighbours = np.asarray(geometry.neighbours)
    normals = np.asarray(geometry.face_normals, dtype=np.float64).reshape(-1, 2)
    fc = np.asarray(geometry.face_centers, dtype=np.float64).reshape(-1, 2)
    centers = np.asarray(geometry.centers, dtype=np.float64).reshape(-1, 2)
    faces = np.asarray(geometry.diffusive_boundary_faces, dtype=np.int64)
    kinds = getattr(geometry, "patch_kinds", {})
    patch_ids = np.asarray(getattr(geometry, "patch_ids", np.zeros(len(owners), dtype=np.int64)))
    walls = {int(f): b for b in getattr(geometry, "wall_thermal_boundaries", ()) for f in b.faces}
    inlet = {}
    for i, f in enumerate(np.asarray(geometry.velocity_inlet_faces)):
        inlet[int(f)] = (1 << 28) | i
    for k, bkind in enumerate(bc["kind"]):
        if bkind in (BC_PRESSURE_INLET, BC_MASS_FLOW_INLET):
            for pos in range(int(bc["offsets"][k]), int(bc["offsets"][k + 1])):
                inlet[int(bc["faces"][pos])] = (2 << 28) | pos
    for i, f in enumerate(np.asarray(geometry.far_field_faces)):
        inlet[int(f)] = (3 << 28) | i
    n = len(faces)
    out = {"faces": faces, "kind": np.zeros(n, dtype=np.int32), "thermal": np.zeros(n, dtype=np.int32),
           "inlet": np.zeros(n, dtype=np.int32), "value": np.zeros(n), "nd": np.zeros(n),
           "ghost": np.zeros((n, 2)), "offset": np.zeros((n, 2))}
    for j, f in enumerate(faces):
        o = int(owners[f])
        nrm = normals[f]
        off = fc[f] - centers[o]
        nd = float(np.dot(off, nrm))
        kind = kinds.get(int(patch_ids[f]), "")
        out["offset"][j] = off
        out["nd"][j] = nd
        out["ghost"][j] = 2.0 * nd * nrm if kind in ("Wall", "Symmetry") else 2.0 * off
        if kind == "Wall":
            w = walls.get(int(f))
            if w is None:
                out["kind"][j] = DIFF_WALL_UNKNOWN
            else:
                no_slip = w.mechanical_condition in ("No-slip", "Prescribed velocity")
                out["kind"][j] = DIFF_WALL_NO_SLIP if no_slip else DIFF_WALL_SLIP
                out["thermal"][j] = 0 if w.condition == "Temperature" else 1
                out["value"][j] = w.value
        elif kind == "Symmetry":
            out["kind"][j] = DIFF_SYMMETRY
        elif int(f) in inlet:
            out["kind"][j] = DIFF_INLET
            out["inlet"][j] = inlet[int(f)]
        else:
            out["kind"][j] = DIFF_OTHER
    interior = np.asarray(geometry.interior_faces, dtype=np.int64)
    o, nb = owners[interior], neighbours[interior]
    out["interior_distance"] = np.abs(np.sum((centers[nb] - centers[o]) * normals[interior], axis=1))
    fa = np.asarray(geometry.periodic_faces_a, dtype=np.int64)
    fb = np.asarray(geometry.periodic_faces_b, dtype=np.int64)
    out["periodic_distance"] = (np.abs(np.sum((fc[fa] - centers[owners[fa]]) * normals[fa], axis=1))
                                + np.abs(np.sum((fc[fb] - centers[owners[fb]]) * normals[fb], axis=1)))
    return out


def _device_view(ptr: int, shape, device) -> torch.Tensor:
    """Wrap a library-owned device buffer (lifetime = the handle)."""
    n = int(np.prod(shape))

    class _Holder:
        __cuda_array_interface__ = {
            "shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 3, "strides": None,
        }

    with torch.cuda.device(device):
        return torch.as_tensor(_Holder(), device=device).view(*shape)
