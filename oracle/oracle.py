"""ORACLE — test infrastructure only (tests, smoke check, CPU baseline).

ctypes wrapper of ``mcfd_oracle.c``, the plain-C restatement of the
reference's residual / time-step / explicit-step path, plus a small driver of
the reference's explicit time loop (``solve_case``, solver.py:437-806) for
multi-step parity runs.  The product never imports this module.
"""

from __future__ import annotations

import ctypes as C
import math
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libmcfd_oracle.so"

FLUX = {"Rusanov": 0, "HLLC": 1, "Roe": 2}
RECON = {"First order": 0, "MUSCL linear": 1, "MUSCL parabolic": 2}
LIMITER = {"Barth-Jespersen": 0, "Minmod": 1, "Van Leer": 2, "Venkatakrishnan": 3, "Venkatakrishnan K": 4}
SCHEME = {"Explicit Euler": 0, "Explicit RK2": 1, "Explicit RK3": 2, "Explicit RK4": 3}

STATUS_TEXT = {
    0x01: "Euler state has non-finite or non-positive density or pressure.",
    0x02: "Spatial residual contains non-finite values.",
    0x04: "HLLC flux produced a non-finite value.",
    0x08: "Roe average has a non-positive sound speed.",
    0x10: "Roe flux produced a non-finite value.",
    0x20: "Far-field characteristics produced invalid sound speed.",
    0x40: "Far-field characteristics produced an invalid state.",
    0x80: "Local stable time steps must be positive and finite.",
    0x100: "Pressure inlet flow direction must point into the domain across every face.",
    0x200: "Pressure inlet cannot prescribe a supersonic outflow.",
    0x400: "Pressure inlet needs Mach number to define a supersonic inflow.",
    0x800: "Pressure inlet total conditions are incompatible with the interior characteristic state.",
    0x1000: "Pressure inlet produced an invalid state.",
    0x2000: "Mass-flow inlet direction must point into the domain across every face.",
    0x4000: "Mass-flow inlet has invalid interior pressure.",
    0x8000: "Mass-flow inlet cannot satisfy the configured flow rate.",
    0x10000: "Mass-flow outlet has invalid interior density.",
}

P64 = C.POINTER(C.c_int64)
PD = C.POINTER(C.c_double)


class OrcGeom(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int64), ("n_faces", C.c_int64),
        ("centers", PD), ("areas", PD), ("face_centers", PD), ("face_normals", PD), ("face_lengths", PD),
        ("wall_velocities", PD), ("owners", P64), ("neighbours", P64),
        ("n_interior", C.c_int64), ("interior_faces", P64),
        ("interior_owner_offsets", PD), ("interior_neighbour_offsets", PD),
        ("n_periodic", C.c_int64), ("periodic_faces_a", P64), ("periodic_faces_b", P64),
        ("n_wall", C.c_int64), ("wall_faces", P64),
        ("n_vin", C.c_int64), ("vin_faces", P64), ("vin_states", PD),
        ("n_pout", C.c_int64), ("pout_faces", P64), ("pout_pressures", PD),
        ("n_far", C.c_int64), ("far_faces", P64), ("far_states", PD),
        ("n_gradient", C.c_int64), ("gradient_sources", P64), ("gradient_neighbours", P64),
        ("gradient_cx", PD), ("gradient_cy", PD),
        ("n_limiter", C.c_int64), ("limiter_cells", P64), ("limiter_dx", PD), ("limiter_dy", PD),
        ("n_parabolic", C.c_int64), ("parabolic_sources", P64), ("parabolic_neighbours", P64),
        ("parabolic_dx", PD), ("parabolic_dy", PD),
        ("n_bc_patches", C.c_int64), ("bc_kind", C.POINTER(C.c_int32)), ("bc_values", PD), ("bc_offsets", P64),
        ("bc_faces", P64), ("bc_dn", PD),
    ]


class OrcSettings(C.Structure):
    _fields_ = [("flux", C.c_int32), ("reconstruction", C.c_int32), ("limiter", C.c_int32), ("pad", C.c_int32),
                ("gamma", C.c_double), ("acceleration_x", C.c_double), ("acceleration_y", C.c_double),
                ("cfl", C.c_double), ("gas_constant", C.c_double), ("venkat_k", C.c_double)]


def build(force: bool = False) -> Path:
    src = HERE / "mcfd_oracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        LIB.parent.mkdir(exist_ok=True)
        subprocess.run(["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-std=c99", "-shared",
                        "-o", str(LIB), str(src), "-lm"], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.orc_residual.argtypes = [C.POINTER(OrcGeom), C.POINTER(OrcSettings), PD, PD]
        _lib.orc_stable_time_steps.argtypes = [C.POINTER(OrcGeom), C.POINTER(OrcSettings), PD, PD, PD]
        _lib.orc_explicit_step.argtypes = [C.POINTER(OrcGeom), C.POINTER(OrcSettings), C.c_int, PD, PD, C.c_int]
        _lib.orc_conservative_to_primitive.argtypes = [C.c_int64, PD, C.c_double, PD]
        _lib.orc_primitive_to_conservative.argtypes = [C.c_int64, PD, C.c_double, PD]
        _lib.orc_linear_gradients_and_factors.argtypes = [C.POINTER(OrcGeom), PD, C.c_int, C.c_double, PD, PD]
        _lib.orc_parabolic_reconstruction.argtypes = [C.POINTER(OrcGeom), PD, C.c_int, PD, PD, PD]
        _lib.orc_bc_states.argtypes = [C.POINTER(OrcGeom), C.c_int64, PD, C.c_double, C.c_double, PD]
        _lib.orc_far_field_states.argtypes = [C.c_int64, PD, PD, PD, C.c_double, PD]
        _lib.orc_face_fluxes.argtypes = [C.c_int, C.c_int64, PD, PD, PD, C.c_double, PD]
        _lib.orc_cell_geometry.argtypes = [C.c_int64, P64, P64, PD, PD, PD, P64]
        _lib.orc_face_geometry.argtypes = [C.c_int64, P64, PD, PD, P64, PD, PD, PD, P64]
    return _lib


class GeometryHost:
    """The cell and face loops of ``_build_geometry`` (solver.py:1654-1696)
    in the oracle's C, with the interface ``build_geometry(..., host=)``
    expects: the CPU reference path builds its mesh geometry with these, so
    it never loads the product library."""

    @staticmethod
    def cell_geometry(offsets, nodes, points):
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        nodes = np.ascontiguousarray(nodes, dtype=np.int64)
        points = np.ascontiguousarray(points, dtype=np.float64)
        n = len(offsets) - 1
        centers, areas, bad = np.empty((n, 2)), np.empty(n), C.c_int64(-1)
        rc = lib().orc_cell_geometry(n, offsets.ctypes.data_as(P64), nodes.ctypes.data_as(P64),
                                     points.ctypes.data_as(PD), centers.ctypes.data_as(PD),
                                     areas.ctypes.data_as(PD), C.byref(bad))
        if rc:
            raise OracleError(f"Cell {bad.value} has zero or invalid area.")
        return centers, areas

    @staticmethod
    def face_geometry(faces, points, centers, owners):
        faces = np.ascontiguousarray(faces, dtype=np.int64)
        points = np.ascontiguousarray(points, dtype=np.float64)
        centers = np.ascontiguousarray(centers, dtype=np.float64)
        owners = np.ascontiguousarray(owners, dtype=np.int64)
        n = len(faces)
        fc, normals, lengths, bad = np.empty((n, 2)), np.empty((n, 2)), np.empty(n), C.c_int64(-1)
        rc = lib().orc_face_geometry(n, faces.ctypes.data_as(P64), points.ctypes.data_as(PD),
                                     centers.ctypes.data_as(PD), owners.ctypes.data_as(P64),
                                     fc.ctypes.data_as(PD), normals.ctypes.data_as(PD),
                                     lengths.ctypes.data_as(PD), C.byref(bad))
        if rc:
            raise OracleError(f"Face {bad.value} has zero or invalid length.")
        return fc, normals, lengths


FACE_FLUXES = {"Rusanov": 0, "HLLC": 1, "Roe": 2, "HLLC kernel": 3}


def face_fluxes(kind, left, right, normals, gamma):
    """The numerical flux ``kind`` (a key of FACE_FLUXES) of rows of left /
    right primitive states (n, 4) across unit normals (n, 2)."""
    left = np.ascontiguousarray(left, dtype=np.float64)
    right = np.ascontiguousarray(right, dtype=np.float64)
    normals = np.ascontiguousarray(normals, dtype=np.float64)
    out = np.empty_like(left)
    _raise(lib().orc_face_fluxes(FACE_FLUXES[kind], len(left), left.ctypes.data_as(PD), right.ctypes.data_as(PD),
                                 normals.ctypes.data_as(PD), gamma, out.ctypes.data_as(PD)))
    return out


def far_field_states(interior, far_field, normals, gamma):
    """_far_field_boundary_states (solver.py:4350-4409): exterior primitive
    states of far-field faces from interior states, far-field states and
    unit normals, each (n, 4) / (n, 2)."""
    interior = np.ascontiguousarray(interior, dtype=np.float64)
    far_field = np.ascontiguousarray(far_field, dtype=np.float64)
    normals = np.ascontiguousarray(normals, dtype=np.float64)
    ext = np.empty_like(interior)
    _raise(lib().orc_far_field_states(len(interior), interior.ctypes.data_as(PD), far_field.ctypes.data_as(PD),
                                      normals.ctypes.data_as(PD), gamma, ext.ctypes.data_as(PD)))
    return ext


class OracleError(ValueError):
    pass


def _raise(code: int):
    for bit, text in STATUS_TEXT.items():
        if code & bit:
            raise OracleError(text)
    if code:
        raise OracleError(f"oracle status {code:#x}")


def _boundary_patches(g):
    """Pressure-inlet / mass-flow patches of a geometry in the reference's
    order, with NumPy's own ``normals @ direction`` (solver.py:4423, 4507) and
    ``np.sum`` of the outlet face lengths (solver.py:4568)."""
    normals = np.asarray(g.face_normals, dtype=np.float64).reshape(-1, 2)
    lengths = np.asarray(g.face_lengths, dtype=np.float64)
    kinds, values, offsets, faces, dn = [], [], [0], [], []
    for kind, patches in ((0, getattr(g, "pressure_inlets", ())), (1, getattr(g, "mass_flow_inlets", ())),
                          (2, getattr(g, "mass_flow_outlets", ()))):
        for b in patches:
            f = np.asarray(b.faces, dtype=np.int64)
            if kind == 2:
                values.append((b.mass_flow, float(np.sum(lengths[f])), 0.0, 0.0))
                dn.append(np.zeros(len(f)))
            else:
                first = b.total_pressure if kind == 0 else b.mass_flow
                values.append((first, b.total_temperature, b.direction[0], b.direction[1]))
                dn.append(normals[f] @ np.asarray(b.direction, dtype=np.float64))
            kinds.append(kind)
            faces.append(f)
            offsets.append(offsets[-1] + len(f))
    cat = (lambda parts, dt: np.ascontiguousarray(np.concatenate(parts), dtype=dt) if parts else np.empty(0, dt))
    return {"kind": np.asarray(kinds, dtype=np.int32), "values": np.ascontiguousarray(values, dtype=np.float64),
            "offsets": np.asarray(offsets, dtype=np.int64), "faces": cat(faces, np.int64), "dn": cat(dn, np.float64)}


class Oracle:
    """Binds one geometry (reference ``_Geometry`` or ``meshcfd_gb300`` Geometry)."""

    def __init__(self, geometry):
        g = geometry
        keep = {}

        def arr(name, dtype, shape=None):
            v = getattr(g, name, None)
            if v is None:
                return None
            a = np.ascontiguousarray(np.asarray(v, dtype=dtype))
            if shape is not None:
                a = a.reshape(shape)
            keep[name] = a
            return a

        def p(a, kind):
            return a.ctypes.data_as(kind) if a is not None and a.size else None

        n_cells = len(g.areas)
        n_faces = len(g.face_lengths)
        fields = dict(
            centers=arr("centers", np.float64, (-1, 2)), areas=arr("areas", np.float64),
            face_centers=arr("face_centers", np.float64, (-1, 2)), face_normals=arr("face_normals", np.float64, (-1, 2)),
            face_lengths=arr("face_lengths", np.float64), wall_velocities=arr("wall_velocities", np.float64, (-1, 2)),
            owners=arr("owners", np.int64), neighbours=arr("neighbours", np.int64),
            interior_faces=arr("interior_faces", np.int64),
            interior_owner_offsets=arr("interior_owner_offsets", np.float64, (-1, 2)),
            interior_neighbour_offsets=arr("interior_neighbour_offsets", np.float64, (-1, 2)),
            periodic_faces_a=arr("periodic_faces_a", np.int64), periodic_faces_b=arr("periodic_faces_b", np.int64),
            wall_faces=arr("wall_faces", np.int64),
            vin_faces=arr("velocity_inlet_faces", np.int64), vin_states=arr("velocity_inlet_states", np.float64, (-1, 4)),
            pout_faces=arr("pressure_outlet_faces", np.int64), pout_pressures=arr("pressure_outlet_pressures", np.float64),
            far_faces=arr("far_field_faces", np.int64), far_states=arr("far_field_states", np.float64, (-1, 4)),
            gradient_sources=arr("gradient_sources", np.int64), gradient_neighbours=arr("gradient_neighbours", np.int64),
            gradient_cx=arr("gradient_coefficients_x", np.float64), gradient_cy=arr("gradient_coefficients_y", np.float64),
            limiter_cells=arr("limiter_cells", np.int64), limiter_dx=arr("limiter_dx", np.float64),
            limiter_dy=arr("limiter_dy", np.float64),
            parabolic_sources=arr("parabolic_sources", np.int64),
            parabolic_neighbours=arr("parabolic_neighbours", np.int64),
            parabolic_dx=arr("parabolic_dx", np.float64), parabolic_dy=arr("parabolic_dy", np.float64),
        )
        s = OrcGeom()
        s.n_cells, s.n_faces = n_cells, n_faces
        for name, a in fields.items():
            kind = P64 if a is not None and a.dtype == np.int64 else PD
            setattr(s, name, p(a, kind))
        s.n_interior = len(fields["interior_faces"])
        s.n_periodic = len(fields["periodic_faces_a"])
        s.n_wall = len(fields["wall_faces"])
        s.n_vin = len(fields["vin_faces"])
        s.n_pout = len(fields["pout_faces"])
        s.n_far = len(fields["far_faces"])
        s.n_gradient = len(fields["gradient_sources"])
        s.n_limiter = len(fields["limiter_cells"])
        s.n_parabolic = 0 if fields["parabolic_sources"] is None else len(fields["parabolic_sources"])
        bc = _boundary_patches(g)
        s.n_bc_patches = len(bc["kind"])
        if s.n_bc_patches:
            keep.update({"bc_" + k: v for k, v in bc.items()})
            s.bc_kind = bc["kind"].ctypes.data_as(C.POINTER(C.c_int32))
            s.bc_values = p(bc["values"], PD)
            s.bc_offsets = p(bc["offsets"], P64)
            s.bc_faces = p(bc["faces"], P64)
            s.bc_dn = p(bc["dn"], PD)
        self.struct = s
        self._keep = keep
        self.n_cells = n_cells
        self.geometry = g
        self._divergence = None

    @staticmethod
    def settings(num) -> OrcSettings:
        s = OrcSettings()
        s.flux = FLUX[num.flux]
        s.reconstruction = RECON[num.reconstruction]
        s.limiter = LIMITER[num.limiter]
        s.gamma = num.gamma
        s.acceleration_x = num.acceleration_x
        s.acceleration_y = num.acceleration_y
        s.cfl = num.cfl
        s.gas_constant = num.gas_constant
        s.venkat_k = float(getattr(num, "venkatakrishnan_k", 5.0))
        return s

    def primitive(self, U, gamma):
        U = np.ascontiguousarray(U, dtype=np.float64)
        P = np.empty_like(U)
        code = lib().orc_conservative_to_primitive(len(U), U.ctypes.data_as(PD), gamma, P.ctypes.data_as(PD))
        _raise(code)
        return P

    def conservative(self, P, gamma):
        P = np.ascontiguousarray(P, dtype=np.float64)
        U = np.empty_like(P)
        lib().orc_primitive_to_conservative(len(P), P.ctypes.data_as(PD), gamma, U.ctypes.data_as(PD))
        return U

    def divergence(self, flux):
        """interior_divergence_operator @ flux (solver.py:2160-2174), SciPy CSR
        as the reference builds it."""
        if self._divergence is None:
            from scipy.sparse import coo_matrix

            g = self.geometry
            faces = np.asarray(g.interior_faces)
            o, n = np.asarray(g.owners)[faces], np.asarray(g.neighbours)[faces]
            L, A = np.asarray(g.face_lengths)[faces], np.asarray(g.areas)
            ids = np.arange(len(faces))
            self._divergence = coo_matrix((np.concatenate((-L / A[o], L / A[n])),
                                           (np.concatenate((o, n)), np.concatenate((ids, ids)))),
                                          shape=(self.n_cells, len(faces))).tocsr()
        return self._divergence @ flux

    def residual(self, U, num):
        U = np.ascontiguousarray(U, dtype=np.float64)
        R = np.empty_like(U)
        viscous = getattr(num, "viscosity_model", "Inviscid") != "Inviscid"
        s = self.settings(num)
        if viscous:  # body force after the viscous terms (solver.py:2699-2715)
            s.acceleration_x = s.acceleration_y = 0.0
        code = lib().orc_residual(C.byref(self.struct), C.byref(s), U.ctypes.data_as(PD), R.ctypes.data_as(PD))
        if not viscous:
            _raise(code)
            return R
        _raise(code & ~0x02)
        from .viscous import viscous_residual

        P = self.primitive(U, num.gamma)
        R = R + viscous_residual(P, self.geometry, num, self, self.divergence)
        ax, ay = num.acceleration_x, num.acceleration_y
        if ax != 0.0 or ay != 0.0:
            R[:, 1] += P[:, 0] * ax
            R[:, 2] += P[:, 0] * ay
            R[:, 3] += P[:, 0] * (ax * P[:, 1] + ay * P[:, 2])
        if not np.isfinite(R).all():
            _raise(0x02)
        return R

    def gradients_and_factors(self, P, limiter, venkat_k=5.0):
        P = np.ascontiguousarray(P, dtype=np.float64)
        grad = np.empty((len(P), 4, 2))
        fac = np.empty((len(P), 4))
        lib().orc_linear_gradients_and_factors(C.byref(self.struct), P.ctypes.data_as(PD), LIMITER[limiter],
                                               float(venkat_k), grad.ctypes.data_as(PD), fac.ctypes.data_as(PD))
        return grad, fac

    def parabolic_reconstruction(self, P, limiter):
        """(gradients (C,4,2), curvature (C,4,3), factors (C,4)) of
        _parabolic_reconstruction (solver.py:2322-2415)."""
        P = np.ascontiguousarray(P, dtype=np.float64)
        grad = np.empty((len(P), 4, 2))
        curv = np.empty((len(P), 4, 3))
        fac = np.empty((len(P), 4))
        lib().orc_parabolic_reconstruction(C.byref(self.struct), P.ctypes.data_as(PD), LIMITER[limiter],
                                           grad.ctypes.data_as(PD), curv.ctypes.data_as(PD), fac.ctypes.data_as(PD))
        return grad, curv, fac

    def boundary_states(self, k, interior, gamma, gas_constant):
        """Exterior states of boundary patch ``k`` (pressure inlets, then
        mass-flow inlets, then outlets) for interior states (n, 4)."""
        interior = np.ascontiguousarray(interior, dtype=np.float64)
        ext = np.empty_like(interior)
        _raise(lib().orc_bc_states(C.byref(self.struct), k, interior.ctypes.data_as(PD), gamma, gas_constant,
                                   ext.ctypes.data_as(PD)))
        return ext

    def stable_time_steps(self, P, num):
        P = np.ascontiguousarray(P, dtype=np.float64)
        dt = np.empty(len(P))
        s = self.settings(num)
        diff = None
        if getattr(num, "viscosity_model", "Inviscid") != "Inviscid":
            from .viscous import diffusion_sum

            diff = np.ascontiguousarray(diffusion_sum(P, self.geometry, num))
        _raise(lib().orc_stable_time_steps(C.byref(self.struct), C.byref(s), P.ctypes.data_as(PD),
                                           diff.ctypes.data_as(PD) if diff is not None else None,
                                           dt.ctypes.data_as(PD)))
        return dt

    def explicit_step(self, U, num, dt):
        if getattr(num, "viscosity_model", "Inviscid") != "Inviscid":
            return self._explicit_step_python(U, num, dt)
        U = np.array(U, dtype=np.float64, order="C", copy=True)
        dt_arr = np.ascontiguousarray(np.atleast_1d(np.asarray(dt, dtype=np.float64)))
        s = self.settings(num)
        code = lib().orc_explicit_step(C.byref(self.struct), C.byref(s), SCHEME[num.time_integration],
                                       U.ctypes.data_as(PD), dt_arr.ctypes.data_as(PD), int(dt_arr.size > 1))
        _raise(code)
        return U

    def _explicit_step_python(self, U, num, dt):
        """The explicit stage combinations (solver.py:532-756) around
        :meth:`residual` (for settings the C step does not cover)."""
        U0 = np.array(U, dtype=np.float64, copy=True)
        d = np.asarray(dt, dtype=np.float64)
        d = d[:, None] if d.ndim == 1 and d.size > 1 else float(d.reshape(-1)[0])
        scheme = SCHEME[num.time_integration]
        if scheme == 3:
            raise NotImplementedError("oracle: viscous SSPRK(5,4) step")
        U1 = U0 + d * self.residual(U0, num)
        if scheme == 0:
            self.primitive(U1, num.gamma)
            return U1
        self.primitive(U1, num.gamma)
        if scheme == 1:
            out = 0.5 * U0 + 0.5 * (U1 + d * self.residual(U1, num))
            self.primitive(out, num.gamma)
            return out
        U2 = 0.75 * U0 + 0.25 * (U1 + d * self.residual(U1, num))
        self.primitive(U2, num.gamma)
        out = (1.0 / 3.0) * U0 + (2.0 / 3.0) * (U2 + d * self.residual(U2, num))
        self.primitive(out, num.gamma)
        return out

    def solve(self, U, num, steps, time=0.0, history=None):
        """The reference's explicit loop (solver.py:437-806) for ``steps`` steps:
        primitive check, time step (global adaptive / fixed / local), one step."""
        U = np.array(U, dtype=np.float64, copy=True)
        for _ in range(steps):
            P = self.primitive(U, num.gamma)
            if num.time_step_mode == "Local (steady)":
                dt = self.stable_time_steps(P, num)
                time_step = float(np.mean(dt))
            elif num.time_step_mode == "Global fixed":
                time_step = min(num.fixed_time_step, num.end_time - time)
                dt = time_step
            else:
                time_step = min(float(np.min(self.stable_time_steps(P, num))), num.end_time - time)
                dt = time_step
            if not math.isfinite(time_step) or time_step <= 0.0:
                raise OracleError("The stable time step is non-positive or non-finite.")
            U = self.explicit_step(U, num, dt)
            time += time_step
            if history is not None:
                history.append((time_step, U.copy()))
        return U, time
