"""Generate the golden fixtures in this folder from the reference itself.

Run from the repository root:  python tests/golden/make_golden.py
(needs a reference checkout, see reference_shim.py).  Each .npz holds the
reference's own geometry arrays (prefixed ``geom_``), the input state and the
reference's outputs, so the tests can run without the reference:

* residual_<case>.npz  — ``_residual`` for every flux x reconstruction x
  limiter combination, with and without a body force, plus
  ``_stable_time_steps``;
* solve_<case>.npz     — final states of ``solve_case`` after N explicit steps;
* bc_<kind>.npz        — ``_residual`` and ``_stable_time_steps`` with
  pressure-inlet or mass-flow inlet / outlet boundaries (plus
  solve_<kind>_rk3.npz);
* parabolic_<case>.npz — ``_residual`` with MUSCL parabolic reconstruction for
  every flux x limiter (with and without a body force) and the outputs of
  ``_parabolic_reconstruction`` per limiter, on a geometry built with the
  two-ring stencil;
* meshio.json          — the reference's MeshCAD JSON reader (io/mesh_io.py) on
  valid inputs (its cell loops and re-serialisation) and its error message
  for each mutation in ``MESH_MUTATIONS``  (mode ``meshio``).
"""

from __future__ import annotations

import itertools
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parents[1]))

from reference_shim import import_reference, reference_case  # noqa: E402

from meshcfd_gb300.meshes import (  # noqa: E402
    bump_case,
    box_mesh,
    cell_centroids,
    ogrid_case,
    periodic_case,
    riemann_case,
    smooth_primitive,
    vortex_case,
    vortex_primitive,
)
from meshcfd_gb300.model import Case  # noqa: E402

GEOM_FIELDS = (
    "centers", "areas", "face_centers", "face_normals", "face_lengths", "wall_velocities", "owners",
    "neighbours", "interior_faces", "interior_owners", "interior_neighbours", "interior_normals",
    "interior_lengths", "interior_owner_offsets", "interior_neighbour_offsets", "wall_faces",
    "symmetry_faces", "periodic_faces_a", "periodic_faces_b", "velocity_inlet_faces",
    "velocity_inlet_states", "pressure_outlet_faces", "pressure_outlet_pressures", "far_field_faces",
    "far_field_states", "gradient_sources", "gradient_neighbours", "gradient_dx", "gradient_dy",
    "gradient_coefficients_x", "gradient_coefficients_y", "limiter_cells", "limiter_dx", "limiter_dy",
)
FLUXES = ("Rusanov", "HLLC", "Roe")
LIMITERS = ("Barth-Jespersen", "Minmod", "Van Leer", "Venkatakrishnan")


def channel_case(nx=7, ny=5):
    mesh = box_mesh(nx, ny, 2.0, 1.0, split="half", jitter=0.2, seed=5)
    case = Case(name="channel", mesh=mesh)
    for c in case.boundary_conditions:
        if c.patch_name == "left":
            c.kind = "Velocity Inlet"
            c.values = {"density": 1.0, "velocity_x": 0.3, "velocity_y": 0.05, "temperature": 1.0 / 287.05}
        elif c.patch_name == "right":
            c.kind = "Pressure Outlet"
            c.values = {"pressure": 0.95}
        elif c.patch_name == "top":
            c.kind = "Symmetry"
        else:
            c.kind = "Wall"
            c.mechanical_condition = "Slip"
    return case


def mesh_arrays(case):
    m = case.mesh
    return {
        "mesh_points": np.asarray(m.points), "mesh_cell_offsets": np.asarray(m.cells.offsets),
        "mesh_cell_nodes": np.asarray(m.cells.nodes), "mesh_faces": np.asarray(m.faces),
        "mesh_face_owners": np.asarray(m.face_owners), "mesh_face_neighbours": np.asarray(m.face_neighbours),
        "mesh_face_patch_ids": np.asarray(m.face_patch_ids),
    }


PARABOLIC_FIELDS = ("parabolic_sources", "parabolic_neighbours", "parabolic_dx", "parabolic_dy")


def geometry_arrays(geometry, fields=GEOM_FIELDS):
    out = {f"geom_{name}": np.asarray(getattr(geometry, name)) for name in fields}
    out.update(bc_patch_arrays(geometry))
    return out


def bc_patch_arrays(geometry):
    """Pressure-inlet / mass-flow patches as flat arrays (kind 0 / 1 / 2;
    values: total p, total T, direction / mass flow, total T, direction /
    mass flow)."""
    kinds, names, values, offsets, faces = [], [], [], [0], []
    for kind, patches in ((0, geometry.pressure_inlets), (1, geometry.mass_flow_inlets),
                          (2, geometry.mass_flow_outlets)):
        for b in patches:
            if kind == 0:
                values.append((b.total_pressure, b.total_temperature, *b.direction))
            elif kind == 1:
                values.append((b.mass_flow, b.total_temperature, *b.direction))
            else:
                values.append((b.mass_flow, 0.0, 0.0, 0.0))
            kinds.append(kind)
            names.append(b.patch_name)
            faces.extend(int(f) for f in b.faces)
            offsets.append(len(faces))
    if not kinds:
        return {}
    return {"bcp_kind": np.asarray(kinds), "bcp_names": np.asarray(names), "bcp_values": np.asarray(values),
            "bcp_offsets": np.asarray(offsets), "bcp_faces": np.asarray(faces, dtype=np.int64)}


def perturbed_primitive(n, seed):
    P = smooth_primitive(n, seed=seed, amplitude=2.0)
    P[:, 1] += 0.3 * np.sin(np.arange(n))
    P[:, 3] *= 1.0 + 0.2 * np.cos(0.7 * np.arange(n))
    return P


def residual_fixture(name, case, ref):
    rc = reference_case(case, ref)
    rg = ref.solver._build_geometry(rc.mesh, rc)
    out = {**mesh_arrays(case), **geometry_arrays(rg)}
    n = len(rg.areas)
    P = perturbed_primitive(n, seed=1)
    U = ref.euler.primitive_to_conservative(P, 1.4)
    out["U"] = U
    num = rc.numerics
    keys = []
    for flux, recon, limiter, force in itertools.product(FLUXES, ("First order", "MUSCL linear"), LIMITERS, (0, 1)):
        if recon == "First order" and limiter != "Barth-Jespersen":
            continue
        num.flux, num.reconstruction, num.limiter = flux, recon, limiter
        num.acceleration_x, num.acceleration_y = (0.3, -0.2) if force else (0.0, 0.0)
        key = f"R|{flux}|{recon}|{limiter}|{force}"
        out[key] = ref.solver._residual(U, rg, num)
        keys.append(key)
    num.acceleration_x = num.acceleration_y = 0.0
    num.cfl = 0.7
    out["dt_cells"] = ref.solver._stable_time_steps(ref.euler.conservative_to_primitive(U, 1.4), rg, num)
    # limiter factors and gradients of the compiled kernels, for every code
    Pp = ref.euler.conservative_to_primitive(U, 1.4)
    for code in range(4):
        g, f = ref.kernels.linear_gradients_and_factors(
            Pp, rg.gradient_sources, rg.gradient_neighbours, rg.gradient_coefficients_x,
            rg.gradient_coefficients_y, rg.limiter_cells, rg.limiter_dx, rg.limiter_dy, code)
        out[f"grad|{code}"] = g
        out[f"factors|{code}"] = f
    out["cfl"] = np.array(0.7)
    np.savez_compressed(HERE / f"residual_{name}.npz", **out)
    print(name, n, "cells,", len(keys), "residuals")


def bc_case(kind, nx=16, ny=9):
    """Jittered half-split channel [0,2]x[0,1] with slip walls top and bottom
    and, left -> right, a pressure inlet -> pressure outlet ("pinlet") or a
    mass-flow inlet -> mass-flow outlet ("massflow"); gas constant 287.05,
    so temperature 1/287.05 means R T = 1.  The reference's mass-flow inlet
    state only works for single-face patches (its velocity array has one row,
    solver.py:4552-4554), so in "massflow" every left face is an inlet patch
    of its own with its share of the flow rate."""
    mesh = box_mesh(nx, ny, 2.0, 1.0, split="half", jitter=0.2, seed=7, separate_left=(kind == "massflow"))
    case = Case(name=kind, mesh=mesh)
    for c in case.boundary_conditions:
        if c.patch_name.startswith("left") and kind == "massflow":
            c.kind = "Mass Flow Inlet"
            c.values = {"mass_flow": 0.3 / ny, "temperature": 1.1 / 287.05, "velocity_x": 1.0, "velocity_y": -0.1}
        elif c.patch_name == "left":
            if kind == "pinlet":
                c.kind = "Pressure Inlet"
                c.values = {"pressure": 1.2, "temperature": 1.1 / 287.05, "velocity_x": 1.0, "velocity_y": 0.2}
            else:
                c.kind = "Mass Flow Inlet"
                c.values = {"mass_flow": 0.3, "temperature": 1.1 / 287.05, "velocity_x": 1.0, "velocity_y": -0.1}
        elif c.patch_name == "right":
            if kind == "pinlet":
                c.kind = "Pressure Outlet"
                c.values = {"pressure": 0.95}
            else:
                c.kind = "Mass Flow Outlet"
                c.values = {"mass_flow": 0.3}
        else:
            c.kind = "Wall"
            c.mechanical_condition = "Slip"
    return case


def bc_primitive(n, seed):
    rng = np.random.default_rng(seed)
    base = np.array([1.0, 0.3, 0.0, 1.0])
    return base + np.array([0.05, 0.05, 0.05, 0.05]) * rng.standard_normal((n, 4))


def bc_fixture(kind, ref):
    """Residuals (3 fluxes x first order / MUSCL linear BJ, Venkatakrishnan /
    MUSCL parabolic Venkatakrishnan), stable time steps and a short RK3 solve
    with pressure-inlet or mass-flow boundaries."""
    case = bc_case(kind)
    case.numerics.reconstruction = "MUSCL parabolic"
    rc = reference_case(case, ref)
    rg = ref.solver._build_geometry(rc.mesh, rc)
    out = {**mesh_arrays(case), **geometry_arrays(rg, GEOM_FIELDS + PARABOLIC_FIELDS)}
    n = len(rg.areas)
    P = bc_primitive(n, seed=5)
    U = ref.euler.primitive_to_conservative(P, 1.4)
    out["U"] = U
    num = rc.numerics
    keys = []
    for flux, (recon, limiter) in itertools.product(FLUXES, (("First order", "Barth-Jespersen"),
                                                             ("MUSCL linear", "Barth-Jespersen"),
                                                             ("MUSCL linear", "Venkatakrishnan"),
                                                             ("MUSCL parabolic", "Venkatakrishnan"))):
        num.flux, num.reconstruction, num.limiter = flux, recon, limiter
        key = f"R|{flux}|{recon}|{limiter}|0"
        out[key] = ref.solver._residual(U, rg, num)
        keys.append(key)
    num.cfl = 0.7
    out["dt_cells"] = ref.solver._stable_time_steps(P, rg, num)
    out["cfl"] = np.array(0.7)
    np.savez_compressed(HERE / f"bc_{kind}.npz", **out)
    print("bc", kind, n, "cells,", len(keys), "residuals")
    solve_fixture(f"{kind}_rk3", bc_case(kind), P,
                  {"flux": "HLLC", "reconstruction": "MUSCL linear", "limiter": "Venkatakrishnan",
                   "time_integration": "Explicit RK3", "cfl": 0.6}, 10, ref)


def viscous_case(kind):
    """Cases for the laminar viscous terms.  "noslip": no-slip walls with
    fixed temperature (bottom) and heat flux (top), velocity inlet, pressure
    outlet, constant viscosity 0.01 (R T = 1 units).  "mixed": slip wall
    with heat flux (top), symmetry (bottom), far field (left), mass-flow
    outlet (right).  "periodic": periodic box in SI units (air at ~300 K)."""
    if kind == "periodic":
        case = periodic_case(8, 6, split="half", jitter=0.25, seed=2)
        case.numerics.viscosity_model = "Sutherland"
        return case
    mesh = box_mesh(16, 9, 2.0, 1.0, split="half", jitter=0.2, seed=11)
    case = Case(name=f"viscous-{kind}", mesh=mesh)
    rt = 1.0 / 287.05
    for c in case.boundary_conditions:
        if kind == "noslip":
            if c.patch_name == "left":
                c.kind = "Velocity Inlet"
                c.values = {"density": 1.0, "velocity_x": 0.3, "velocity_y": 0.05, "temperature": rt}
            elif c.patch_name == "right":
                c.kind = "Pressure Outlet"
                c.values = {"pressure": 0.95}
            elif c.patch_name == "bottom":
                c.kind, c.mechanical_condition, c.thermal_condition = "Wall", "No-slip", "Temperature"
                c.values = {"temperature": 1.1 * rt}
            else:
                c.kind, c.mechanical_condition, c.thermal_condition = "Wall", "No-slip", "Heat Flux"
                c.values = {"heat_flux": 0.02}
        else:
            if c.patch_name == "left":
                c.kind = "Far Field"
                c.values = {"density": 1.0, "velocity_x": 0.3, "velocity_y": 0.0, "pressure": 1.0}
            elif c.patch_name == "right":
                c.kind = "Mass Flow Outlet"
                c.values = {"mass_flow": 0.3}
            elif c.patch_name == "bottom":
                c.kind = "Symmetry"
            else:
                c.kind, c.mechanical_condition, c.thermal_condition = "Wall", "Slip", "Heat Flux"
                c.values = {"heat_flux": -0.01}
    case.numerics.viscosity_model = "Constant"
    case.numerics.dynamic_viscosity = 0.01
    return case


def viscous_primitive(kind, n, seed):
    if kind == "periodic":  # air near 300 K
        rng = np.random.default_rng(seed)
        base = np.array([1.2, 30.0, -10.0, 1.2 * 287.05 * 300.0])
        return base * (1.0 + 0.05 * rng.standard_normal((n, 4)))
    return bc_primitive(n, seed)


def viscous_fixture(kind, ref):
    case = viscous_case(kind)
    case.numerics.reconstruction = "MUSCL parabolic"
    rc = reference_case(case, ref)
    rg = ref.solver._build_geometry(rc.mesh, rc)
    out = {**mesh_arrays(case), **geometry_arrays(rg, GEOM_FIELDS + PARABOLIC_FIELDS
                                                  + ("diffusive_boundary_faces", "patch_ids"))}
    out.update(viscous_geometry_arrays(rg))
    n = len(rg.areas)
    P = viscous_primitive(kind, n, seed=5)
    U = ref.euler.primitive_to_conservative(P, 1.4)
    out["U"] = U
    num = rc.numerics
    out["dynamic_viscosity"] = np.array(num.dynamic_viscosity)
    # the wall cases run in R T = 1 units, where Sutherland's law (fit to air
    # in kelvin) does not apply; the periodic box is in SI units
    models = ("Sutherland", "Constant") if kind == "periodic" else ("Constant",)
    keys = []
    for model in models:
        num.viscosity_model = model
        out[f"V|{model}"] = ref.solver._viscous_residual(P, rg, num)
        out[f"G|{model}"] = ref.solver._viscous_gradients(P, rg, num)
        for flux, (recon, limiter) in itertools.product(FLUXES, (("First order", "Barth-Jespersen"),
                                                                 ("MUSCL linear", "Venkatakrishnan"))):
            num.flux, num.reconstruction, num.limiter = flux, recon, limiter
            key = f"R|{flux}|{recon}|{limiter}|0|{model}"
            out[key] = ref.solver._residual(U, rg, num)
            keys.append(key)
        num.cfl = 0.7
        out[f"dt|{model}"] = ref.solver._stable_time_steps(P, rg, num)
    np.savez_compressed(HERE / f"viscous_{kind}.npz", **out)
    print("viscous", kind, n, "cells,", len(keys), "residuals")


def viscous_geometry_arrays(rg):
    """Wall thermal data and patch kinds of a reference geometry."""
    faces, offsets, cond, values, mech, names = [], [0], [], [], [], []
    for b in rg.wall_thermal_boundaries:
        faces.extend(int(f) for f in b.faces)
        offsets.append(len(faces))
        cond.append(b.condition)
        values.append(b.value)
        mech.append(b.mechanical_condition)
        names.append(b.patch_name)
    kinds = sorted(rg.patch_kinds.items())
    return {"wt_faces": np.asarray(faces, dtype=np.int64), "wt_offsets": np.asarray(offsets),
            "wt_condition": np.asarray(cond), "wt_value": np.asarray(values, dtype=float),
            "wt_mechanical": np.asarray(mech), "wt_names": np.asarray(names),
            "patch_kind_ids": np.asarray([k for k, _ in kinds]), "patch_kind_names": np.asarray([v for _, v in kinds])}


def strip_case(nx=6, ny=2):
    """Unsplit, unjittered 6x2 quads: every two-ring stencil has two rows of
    cell centres, so every 5x5 normal matrix is rank deficient."""
    mesh = box_mesh(nx, ny, 3.0, 1.0, split="none", jitter=0.0, seed=0)
    case = channel_case()
    case.mesh = mesh
    return case


def parabolic_fixture(name, case, ref):
    case.numerics.reconstruction = "MUSCL parabolic"
    rc = reference_case(case, ref)
    rg = ref.solver._build_geometry(rc.mesh, rc)
    out = {**mesh_arrays(case), **geometry_arrays(rg, GEOM_FIELDS + PARABOLIC_FIELDS)}
    n = len(rg.areas)
    P = perturbed_primitive(n, seed=1)
    U = ref.euler.primitive_to_conservative(P, 1.4)
    out["U"] = U
    num = rc.numerics
    keys = []
    for flux, limiter, force in itertools.product(FLUXES, LIMITERS, (0, 1)):
        num.flux, num.limiter = flux, limiter
        num.acceleration_x, num.acceleration_y = (0.3, -0.2) if force else (0.0, 0.0)
        key = f"R|{flux}|MUSCL parabolic|{limiter}|{force}"
        out[key] = ref.solver._residual(U, rg, num)
        keys.append(key)
    Pp = ref.euler.conservative_to_primitive(U, 1.4)
    for code, limiter in enumerate(LIMITERS):
        g, k, f = ref.solver._parabolic_reconstruction(Pp, rg, limiter)
        out[f"pgrad|{code}"], out[f"pcurv|{code}"], out[f"pfactors|{code}"] = g, k, f
    np.savez_compressed(HERE / f"parabolic_{name}.npz", **out)
    print("parabolic", name, n, "cells,", len(rg.parabolic_sources), "stencil entries,", len(keys), "residuals")


def solve_fixture(name, case, primitive, settings, steps, ref):
    rc = reference_case(case, ref)
    for key, value in settings.items():
        setattr(rc.numerics, key, value)
    rc.numerics.max_iterations = steps
    rc.numerics.end_time = 1.0e30
    rc.numerics.residual_tolerance = 1e-300
    rc.numerics.convergence_history_interval = steps + 1
    rg = ref.solver._build_geometry(rc.mesh, rc)
    states = tuple(ref.model.InitialState(*map(float, row)) for row in primitive)
    result = ref.solver.solve_case(rc, states)
    final = np.array([(s.density, s.velocity_x, s.velocity_y, s.pressure) for s in result.states])
    fields = GEOM_FIELDS + (PARABOLIC_FIELDS if rc.numerics.reconstruction == "MUSCL parabolic" else ())
    viscous = rc.numerics.viscosity_model != "Inviscid"
    if viscous:
        fields = fields + ("diffusive_boundary_faces", "patch_ids")
    out = {**mesh_arrays(case), **geometry_arrays(rg, fields), "P0": primitive, "P_final": final,
           **(viscous_geometry_arrays(rg) if viscous else {}),
           "time": np.array(result.time), "steps": np.array(result.steps)}
    for key, value in settings.items():
        out[f"set|{key}"] = np.array(value)
    np.savez_compressed(HERE / f"solve_{name}.npz", **out)
    print(name, len(primitive), "cells,", result.steps, "steps, t =", result.time)


def implicit_fixture(name, case, primitive, settings, steps, ref):
    """Implicit Euler: the LU-SGS preconditioner and the finite-difference
    operator applied to seeded vectors, and solve_case after ``steps`` steps."""
    from dataclasses import replace

    rc = reference_case(case, ref)
    for key, value in settings.items():
        setattr(rc.numerics, key, value)
    num = rc.numerics
    rg = ref.solver._build_geometry(rc.mesh, rc)
    out = {**mesh_arrays(case), **geometry_arrays(rg), "P0": primitive}
    n = len(primitive)
    U = ref.euler.primitive_to_conservative(primitive, num.gamma)
    dt = ref.solver._stable_time_steps(primitive, rg, num)
    first = replace(num, reconstruction="First order")
    rng = np.random.default_rng(11)
    v = rng.standard_normal(4 * n)
    M = ref.solver._implicit_preconditioner(primitive, rg, first, dt, 4)
    out.update(U=U, dt_cells=dt, v=v, lusgs_v=M.matvec(v))
    rho = max(float(np.max(primitive[:, 0])), 1e-12)
    speed = max(float(np.max(np.abs(primitive[:, 1:3]))),
                float(np.max(np.sqrt(num.gamma * primitive[:, 3] / primitive[:, 0]))), 1e-12)
    scales = np.maximum(np.max(np.abs(U), axis=0), 1e-12)
    scales[0] = max(scales[0], rho)
    scales[1:3] = np.maximum(scales[1:3], rho * speed)
    scales[3] = max(scales[3], rho * speed**2, float(np.max(primitive[:, 3])) / (num.gamma - 1.0))
    scale_grid = scales[None, :]
    rate = ref.solver._time_state_rhs(U, rg, first)
    op = ref.solver._matrix_free_implicit_operator(U, rate, scale_grid, dt, rg, first)
    out.update(scales=scales, operator_v=op.matvec(v))
    num.max_iterations = steps
    num.end_time = 1.0e30
    num.residual_tolerance = 1e-300
    num.convergence_history_interval = steps + 1
    states = tuple(ref.model.InitialState(*map(float, row)) for row in primitive)
    result = ref.solver.solve_case(rc, states)
    out["P_final"] = np.array([(s.density, s.velocity_x, s.velocity_y, s.pressure) for s in result.states])
    out["time"] = np.array(result.time)
    out["steps"] = np.array(result.steps)
    for key, value in settings.items():
        out[f"set|{key}"] = np.array(value)
    np.savez_compressed(HERE / f"implicit_{name}.npz", **out)
    print("implicit", name, n, "cells,", result.steps, "steps, t =", result.time)


# ------------------------------------------------------------ MeshCAD JSON

def meshio_square():
    """The one-cell unit square of the reference's reader test
    (tests/test_mesh_io.py:6-28)."""
    return {
        "format": "meshcad-mesh", "version": 1, "dimension": 2,
        "nodes": {"coordinates": [[0, 0], [1, 0], [1, 1], [0, 1]]},
        "faces": {"nodes": [[0, 1], [1, 2], [2, 3], [3, 0]], "owner": [0, 0, 0, 0], "patch": [0, 1, 2, 3],
                  "neighbour": [-1, -1, -1, -1]},
        "cells": {"faces": [[0, 1, 2, 3]], "face_signs": [[1, 1, 1, 1]]},
        "patches": [{"id": 0, "name": "bottom", "faces": [0]}, {"id": 1, "name": "right", "faces": [1]},
                    {"id": 2, "name": "top", "faces": [2]}, {"id": 3, "name": "left", "faces": [3]}],
    }


def meshio_pair():
    """Two triangles of the unit square sharing the diagonal (face 2)."""
    return {
        "format": "meshcad-mesh", "version": 1, "dimension": 2,
        "nodes": {"coordinates": [[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]]},
        "faces": {"nodes": [[0, 1], [1, 2], [2, 0], [2, 3], [3, 0]], "owner": [0, 0, 0, 1, 1],
                  "patch": [0, 1, -1, 2, 3], "neighbour": [-1, -1, 1, -1, -1]},
        "cells": {"faces": [[0, 1, 2], [2, 3, 4]], "face_signs": [[1, 1, 1], [-1, 1, 1]]},
        "patches": [{"id": 0, "name": "bottom", "faces": [0]}, {"id": 1, "name": "right", "faces": [1]},
                    {"id": 2, "name": "top", "faces": [3]}, {"id": 3, "name": "left", "faces": [4]}],
    }


def meshio_pair_with_metadata():
    """meshio_pair with line / spline / spline-segment boundary curves and
    refinement metadata."""
    d = meshio_pair()
    d["boundary_curves"] = [
        {"geometry": {"type": "line", "start": [0.0, 0.0], "end": [1.0, 0.0]}, "parameters": [0.0, 1.0],
         "patch_id": 0},
        {"geometry": {"type": "spline", "points": [[1.0, 0.0], [1.1, 0.5], [1.0, 1.0]]}, "parameters": [0.0, 1.0],
         "patch_id": 1},
        None,
        {"geometry": {"type": "spline_segment", "points": [[2.0, 1.0], [1.0, 1.0], [0.0, 1.0], [-1.0, 1.0]],
                      "start_t": 1.0 / 3.0, "end_t": 2.0 / 3.0}, "parameters": [0.0, 1.0], "patch_id": 2},
        {"geometry": {"type": "line", "start": [0.0, 1.0], "end": [0.0, 0.0]}, "parameters": [0.0, 1.0],
         "patch_id": 3},
    ]
    d["refinement"] = {"cell_ids": ["c0", "c1"], "cell_levels": [1, 1],
                       "records": [{"parent_id": "p", "child_ids": ["c0", "c1"],
                                    "vertices": [[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]], "level": 0}]}
    return d


def meshio_figure8(face_order=(0, 1, 2, 3, 4, 5)):
    """One cell made of two triangles that share node 0 (node 0 starts two of
    its edges, so the loop follows the reference's first-match rule)."""
    coords = [[0.0, 0.0], [1.0, 0.0], [0.5, 1.0], [-1.0, 0.0], [-0.5, -1.0]]
    nodes = [[0, 1], [1, 2], [2, 0], [0, 3], [3, 4], [4, 0]]
    return {
        "format": "meshcad-mesh", "version": 1, "dimension": 2,
        "nodes": {"coordinates": coords},
        "faces": {"nodes": nodes, "owner": [0] * 6, "patch": [0] * 6, "neighbour": [-1] * 6},
        "cells": {"faces": [list(face_order)], "face_signs": [[1] * 6]},
        "patches": [{"id": 0, "name": "outer", "faces": list(range(6))}],
    }


def _arc_curve():
    return {"geometry": {"type": "arc", "center": [0.5, 0.5], "radius": 2 ** 0.5 / 2,
                         "start_angle": -3 * 3.141592653589793 / 4, "end_angle": -3.141592653589793 / 4},
            "parameters": [0.0, 1.0], "patch_id": 0}


def _set(path, value):
    def apply(d):
        target = d
        for key in path[:-1]:
            target = target[key]
        target[path[-1]] = value
    return apply


def _delete(path):
    def apply(d):
        target = d
        for key in path[:-1]:
            target = target[key]
        del target[path[-1]]
    return apply


def _append(path, value):
    def apply(d):
        target = d
        for key in path:
            target = target[key]
        target.append(value)
    return apply


def _curves(face, curve, n=4):
    def apply(d):
        curves = [None] * n
        curves[face] = curve
        d["boundary_curves"] = curves
    return apply


def _curve_geometry_set(key, value, base=None):
    def apply(d):
        curve = base() if base else _arc_curve()
        if key in ("parameters", "patch_id"):
            curve[key] = value
        else:
            curve["geometry"][key] = value
        d["boundary_curves"] = [curve, None, None, None]
    return apply


def _line_curve():
    return {"geometry": {"type": "line", "start": [0.0, 0.0], "end": [1.0, 0.0]}, "parameters": [0.0, 1.0],
            "patch_id": 0}


def _spline_segment_curve():
    return {"geometry": {"type": "spline_segment", "points": [[-1.0, 0.0], [0.0, 0.0], [1.0, 0.0], [2.0, 0.0]],
                         "start_t": 1.0 / 3.0, "end_t": 2.0 / 3.0}, "parameters": [0.0, 1.0], "patch_id": 0}


_REC = {"parent_id": "p", "child_ids": ["a", "b"], "vertices": [[0, 0], [1, 0], [0, 1]], "level": 0}

# (name, base mesh, mutation): every branch of the reader's validation
MESH_MUTATIONS = [
    ("format", "square", _set(["format"], "mesh")),
    ("version", "square", _set(["version"], 2)),
    ("dimension", "square", _set(["dimension"], 3)),
    ("missing_nodes", "square", _delete(["nodes"])),
    ("nodes_not_object", "square", _set(["nodes"], [])),
    ("missing_patches", "square", _delete(["patches"])),
    ("no_nodes", "square", _set(["nodes", "coordinates"], [])),
    ("node_shape", "square", _set(["nodes", "coordinates", 1], [1])),
    ("node_text", "square", _set(["nodes", "coordinates", 1], [1, "x"])),
    ("node_nan", "square", _set(["nodes", "coordinates", 0, 0], float("nan"))),
    ("node_inf", "square", _set(["nodes", "coordinates", 2, 1], float("inf"))),
    ("no_faces", "square", _set(["faces", "nodes"], [])),
    ("face_shape", "square", _set(["faces", "nodes", 1], [1, 2, 3])),
    ("face_float", "square", _set(["faces", "nodes", 1], [1, 2.0])),
    ("face_bool", "square", _set(["faces", "nodes", 1], [True, 2])),
    ("face_same_nodes", "square", _set(["faces", "nodes", 1], [1, 1])),
    ("face_node_range", "square", _set(["faces", "nodes", 1], [1, 9])),
    ("face_node_negative", "square", _set(["faces", "nodes", 2], [-1, 2])),
    ("owners_not_list", "square", _set(["faces", "owner"], 3)),
    ("owner_float", "square", _set(["faces", "owner", 0], 0.0)),
    ("neighbour_bool", "square", _set(["faces", "neighbour", 0], False)),
    ("patch_id_text", "square", _set(["faces", "patch", 0], "0")),
    ("face_lengths", "square", _append(["faces", "owner"], 0)),
    ("patches_not_list", "square", _set(["patches"], {})),
    ("patch_not_object", "square", _set(["patches", 0], 5)),
    ("patch_id_missing", "square", _delete(["patches", 0, "id"])),
    ("patch_name_blank", "square", _set(["patches", 0, "name"], " ")),
    ("patch_duplicate_id", "square", _set(["patches", 1, "id"], 0)),
    ("patch_duplicate_name", "square", _set(["patches", 1, "name"], "bottom")),
    ("patch_faces_not_list", "square", _set(["patches", 0, "faces"], 0)),
    ("patch_face_range", "square", _set(["patches", 0, "faces"], [9])),
    ("cells_not_list", "square", _set(["cells", "faces"], {})),
    ("cells_empty", "square", lambda d: d["cells"].update({"faces": [], "face_signs": []})),
    ("cells_signs_length", "square", _append(["cells", "face_signs"], [1, 1, 1])),
    ("unknown_patch", "square", _set(["faces", "patch", 0], 7)),
    ("owner_range", "square", _set(["faces", "owner", 0], 5)),
    ("neighbour_is_owner", "pair", _set(["faces", "neighbour", 2], 0)),
    ("neighbour_range", "pair", _set(["faces", "neighbour", 2], 4)),
    ("boundary_inconsistent", "pair", _set(["faces", "patch", 2], 0)),
    ("cell_faces_not_list", "square", _set(["cells", "faces", 0], 5)),
    ("cell_face_float", "square", _set(["cells", "faces", 0, 0], 0.0)),
    ("cell_two_faces", "square", lambda d: d["cells"].update({"faces": [[0, 1]], "face_signs": [[1, 1]]})),
    ("cell_face_range", "square", _set(["cells", "faces", 0, 0], 9)),
    ("cell_sign", "square", _set(["cells", "face_signs", 0, 0], 2)),
    ("open_cell", "square", _set(["cells", "face_signs", 0, 3], -1)),
    ("second_cell_open", "pair", _set(["cells", "face_signs", 1, 0], 1)),
    ("patch_unrelated_face", "square", _set(["patches", 0, "faces"], [1])),
    ("patch_face_twice", "square", _set(["patches", 0, "faces"], [0, 0])),
    ("patch_membership", "square", _set(["patches", 0, "faces"], [])),
    ("refinement_not_object", "square", _set(["refinement"], [])),
    ("refinement_ids_not_list", "square", _set(["refinement"], {"cell_ids": "a"})),
    ("refinement_id_empty", "square", _set(["refinement"], {"cell_ids": [""]})),
    ("refinement_level_float", "square", _set(["refinement"], {"cell_ids": ["a"], "cell_levels": [0.5]})),
    ("refinement_lengths", "square", _set(["refinement"], {"cell_ids": ["a", "b"], "cell_levels": [0, 0]})),
    ("refinement_negative", "square", _set(["refinement"], {"cell_ids": ["a"], "cell_levels": [-1]})),
    ("records_not_list", "square", _set(["refinement"], {"cell_ids": ["a"], "cell_levels": [0], "records": {}})),
    ("records_need_ids", "square", _set(["refinement"], {"records": [{}]})),
    ("record_not_object", "square", _set(["refinement"], {"cell_ids": ["a"], "cell_levels": [0], "records": [5]})),
    ("record_level_float", "square", _set(["refinement"], {"cell_ids": ["a"], "cell_levels": [0],
                                                           "records": [dict(_REC, level=0.5)]})),
    ("record_one_child", "square", _set(["refinement"], {"cell_ids": ["a"], "cell_levels": [0],
                                                         "records": [dict(_REC, child_ids=["a"])]})),
    ("record_vertex_shape", "square", _set(["refinement"], {"cell_ids": ["a"], "cell_levels": [0],
                                                            "records": [dict(_REC, vertices=[[0, 0], [1, 0], [0]])]})),
    ("record_vertex_nan", "square", _set(["refinement"], {"cell_ids": ["a"], "cell_levels": [0],
                                                          "records": [dict(_REC, vertices=[[0, 0], [1, 0], [float("nan"), 1]])]})),
    ("curves_length", "square", _set(["boundary_curves"], [None])),
    ("curve_not_object", "square", _set(["boundary_curves"], [5, None, None, None])),
    ("curve_on_internal_face", "pair", _curves(2, _line_curve(), 5)),
    ("curve_patch", "square", _curve_geometry_set("patch_id", 1)),
    ("curve_one_parameter", "square", _curve_geometry_set("parameters", [0.0])),
    ("curve_parameter_range", "square", _curve_geometry_set("parameters", [0.0, 2.0])),
    ("curve_equal_parameters", "square", _curve_geometry_set("parameters", [0.5, 0.5])),
    ("curve_type", "square", _curve_geometry_set("type", "circle")),
    ("curve_arc_center", "square", _curve_geometry_set("center", [0])),
    ("curve_arc_radius", "square", _curve_geometry_set("radius", -1.0)),
    ("curve_arc_angle", "square", _curve_geometry_set("start_angle", "x")),
    ("curve_line_start", "square", _curve_geometry_set("start", [0.0], _line_curve)),
    ("curve_spline_points", "square", _curve_geometry_set("points", [[0.0, 0.0]], _spline_segment_curve)),
    ("curve_spline_parameters", "square", _curve_geometry_set("end_t", 0.2, _spline_segment_curve)),
    ("curve_spline_offset", "square", _curve_geometry_set("start_offset", [0.0], _spline_segment_curve)),
    ("curve_mismatch", "square", _curve_geometry_set("parameters", [0.0, 0.5])),
]

MESHIO_BASES = {"square": meshio_square, "pair": meshio_pair}


def meshio_valid_inputs():
    from meshcfd_gb300 import mesh_io

    square_arc = meshio_square()
    square_arc["boundary_curves"] = [_arc_curve(), None, None, None]
    vortex, _ = vortex_case(12, seed=0, jitter=0.15, split="half")
    return {
        "square": meshio_square(),
        "square_arc": square_arc,
        "pair": meshio_pair(),
        "pair_metadata": meshio_pair_with_metadata(),
        "figure8": meshio_figure8(),
        "figure8_scrambled": meshio_figure8((3, 0, 4, 1, 5, 2)),
        "vortex12": mesh_io.mesh_to_dict(vortex.mesh),
    }


def meshio_main():
    """tests/golden/meshio.json: for each valid input the reference reader's
    cell loops and re-serialisation; for each mutation of a valid input the
    reference reader's error message."""
    import copy
    import json

    from reference_shim import import_reference_mesh_io

    ref = import_reference_mesh_io()
    valid = {}
    for name, data in meshio_valid_inputs().items():
        mesh = ref.mesh_from_dict(copy.deepcopy(data))
        valid[name] = {"data": data, "cells": [list(c) for c in mesh.cells], "to_dict": ref.mesh_to_dict(mesh)}
    errors = {}
    for name, base, mutate in MESH_MUTATIONS:
        data = MESHIO_BASES[base]()
        mutate(data)
        try:
            ref.mesh_from_dict(data)
        except ref.MeshImportError as error:
            errors[name] = str(error)
        else:
            raise RuntimeError(f"mutation {name} was accepted by the reference")
    (HERE / "meshio.json").write_text(json.dumps({"valid": valid, "errors": errors}, allow_nan=True))


def main(only=None):
    if only == "meshio":
        return meshio_main()
    ref = import_reference()
    if only == "parabolic":
        return parabolic_main(ref)
    if only == "viscous":
        for kind in ("noslip", "mixed", "periodic"):
            viscous_fixture(kind, ref)
        case = viscous_case("noslip")
        solve_fixture("viscous_noslip_rk3", case, viscous_primitive("noslip", len(case.mesh.cells), 5),
                      {"flux": "HLLC", "reconstruction": "MUSCL linear", "limiter": "Venkatakrishnan",
                       "time_integration": "Explicit RK3", "cfl": 0.5, "viscosity_model": "Constant",
                       "dynamic_viscosity": 0.01}, 10, ref)
        return None
    if only == "bc":
        bc_fixture("pinlet", ref)
        bc_fixture("massflow", ref)
        return None
    if only == "bump":  # the implicit configuration's mesh recipe: slip wall, far field, pressure outlet
        residual_fixture("bump", bump_case(16, 8)[0], ref)
        return None
    if only == "ogrid":  # the adjoint configuration's mesh recipe: curved slip wall, far field
        residual_fixture("ogrid", ogrid_case(32, 16)[0], ref)
        return None
    if only == "fluxes":
        return fluxes_fixture(ref)
    if only == "bump_implicit":
        return bump_implicit_fixture(ref)
    riemann, riemann_p = riemann_case(16)
    residual_fixture("riemann16", riemann, ref)
    residual_fixture("periodic_mixed", periodic_case(8, 6, split="half", jitter=0.25, seed=2), ref)
    residual_fixture("channel", channel_case(), ref)

    solve_fixture("riemann16_euler", riemann, riemann_p,
                  {"flux": "Rusanov", "reconstruction": "First order", "time_integration": "Explicit Euler",
                   "cfl": 0.5}, 40, ref)
    vortex, _ = vortex_case(12, seed=0, jitter=0.15, split="half")
    vp = vortex_primitive(cell_centroids(vortex.mesh))
    solve_fixture("vortex12_rk3", vortex, vp,
                  {"flux": "HLLC", "reconstruction": "MUSCL linear", "limiter": "Venkatakrishnan",
                   "time_integration": "Explicit RK3", "cfl": 0.8}, 12, ref)
    chan = channel_case()
    cp = perturbed_primitive(len(chan.mesh.cells), seed=3)
    cp[:, 0] = np.abs(cp[:, 0])
    solve_fixture("channel_rk4_local", chan, cp,
                  {"flux": "Roe", "reconstruction": "MUSCL linear", "limiter": "Barth-Jespersen",
                   "time_integration": "Explicit RK4", "cfl": 0.6, "time_step_mode": "Local (steady)"}, 6, ref)
    implicit_fixture("channel", chan, cp,
                     {"flux": "Roe", "reconstruction": "MUSCL linear", "limiter": "Barth-Jespersen",
                      "time_integration": "Implicit Euler", "time_step_mode": "Local (steady)", "cfl": 50.0,
                      "gmres_tolerance": 1e-3, "gmres_krylov_dimension": 30, "implicit_preconditioner": "LU-SGS"},
                     4, ref)
    per = periodic_case(8, 6, split="half", jitter=0.25, seed=2)
    pp = perturbed_primitive(len(per.mesh.cells), seed=4)
    pp[:, 0] = np.abs(pp[:, 0])
    implicit_fixture("periodic", per, pp,
                     {"flux": "Rusanov", "reconstruction": "First order", "time_integration": "Implicit Euler",
                      "time_step_mode": "Global adaptive", "cfl": 20.0, "gmres_tolerance": 1e-6,
                      "gmres_krylov_dimension": 10, "implicit_preconditioner": "LU-SGS"}, 3, ref)
    solve_fixture("channel_rk2_vanleer", chan, cp,
                  {"flux": "HLLC", "reconstruction": "MUSCL linear", "limiter": "Van Leer",
                   "time_integration": "Explicit RK2", "cfl": 0.6, "acceleration_x": 0.2}, 8, ref)


def bump_implicit_fixture(ref, nx=16, ny=8):
    """One implicit-Euler step of the reference (_implicit_euler_step) on the
    bump-channel recipe from the free stream with its local time steps:
    at CFL 200 its Newton solve fails until the step has been halved 9
    times, which the fixture records with the new state."""
    case, P = bump_case(nx, ny)
    rc = reference_case(case, ref)
    rg = ref.solver._build_geometry(rc.mesh, rc)
    num = rc.numerics
    U = ref.euler.primitive_to_conservative(P, num.gamma)
    dt = ref.solver._stable_time_steps(ref.euler.conservative_to_primitive(U, num.gamma), rg, num)
    out, used = ref.solver._implicit_euler_step(U, dt, rg, num)
    np.savez_compressed(HERE / "implicit_bump.npz", U=U, dt=dt, U_next=out, used=np.asarray(used))
    print("bump implicit", len(U), "cells, accepted / initial step", float(np.mean(used) / np.mean(dt)))


def fluxes_fixture(ref, n=1000, seed=11):
    """The reference's numerical fluxes (euler.numerical_flux) of random
    face states: subsonic and supersonic, both directions, random unit
    normals."""
    rng = np.random.default_rng(seed)

    def states():
        return np.column_stack((rng.uniform(0.3, 2.0, n), rng.uniform(-3.0, 3.0, n), rng.uniform(-3.0, 3.0, n),
                                rng.uniform(0.3, 2.0, n)))

    L, R = states(), states()
    theta = rng.uniform(0.0, 2.0 * np.pi, n)
    N = np.column_stack((np.cos(theta), np.sin(theta)))
    out = {"L": L, "R": R, "normals": N}
    for kind in ("Rusanov", "HLLC", "Roe"):
        out[kind] = ref.euler.numerical_flux(L, R, N, 1.4, kind)
    np.savez_compressed(HERE / "fluxes.npz", **out)
    print("fluxes", n, "faces")


def parabolic_main(ref):
    riemann, _ = riemann_case(16)
    parabolic_fixture("riemann16", riemann, ref)
    parabolic_fixture("periodic_mixed", periodic_case(8, 6, split="half", jitter=0.25, seed=2), ref)
    parabolic_fixture("channel", channel_case(), ref)
    parabolic_fixture("strip", strip_case(), ref)
    vortex, _ = vortex_case(12, seed=0, jitter=0.15, split="half")
    vp = vortex_primitive(cell_centroids(vortex.mesh))
    solve_fixture("vortex12_rk3_parabolic", vortex, vp,
                  {"flux": "HLLC", "reconstruction": "MUSCL parabolic", "limiter": "Venkatakrishnan",
                   "time_integration": "Explicit RK3", "cfl": 0.8}, 8, ref)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
