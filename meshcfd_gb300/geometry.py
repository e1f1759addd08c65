"""Host-side geometry precompute: the arrays the device residual consumes.

This restates the reference's ``_build_geometry`` (``src/meshcfd/core/solver.py:
1654-2238``) for the boundary kinds on the hot path, producing an object whose
attribute names match the reference ``_Geometry`` (solver.py:123-177).  Either a
reference ``_Geometry`` or a :class:`Geometry` from :func:`build_geometry` can be
handed to :class:`meshcfd_gb300.device.DeviceGeometry`.

Per-cell and per-face loops (shoelace areas, face normals) run in the native
library, with the reference's operation order, so the arrays match the
reference bit for bit on the machine the reference runs on (the face-length norm
there is an FMA-based BLAS dot: ``sqrt(fma(ey, ey, ex*ex))``).  Everything else
is vectorised NumPy with the reference's expression order.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .errors import SolverError
from .model import FiniteVolumeMesh

SUPPORTED_KINDS = (
    "Periodic",
    "Wall",
    "Symmetry",
    "Velocity Inlet",
    "Pressure Inlet",
    "Pressure Outlet",
    "Mass Flow Inlet",
    "Mass Flow Outlet",
    "Far Field",
)


@dataclass(frozen=True)
class PressureInlet:
    """Mirror of ``_PressureInlet`` (solver.py:81-87)."""

    faces: np.ndarray
    total_pressure: float
    total_temperature: float
    direction: np.ndarray
    patch_name: str


@dataclass(frozen=True)
class MassFlowInlet:
    """Mirror of ``_MassFlowInlet`` (solver.py:90-96)."""

    faces: np.ndarray
    mass_flow: float
    total_temperature: float
    direction: np.ndarray
    patch_name: str


@dataclass(frozen=True)
class WallThermalBoundary:
    """Mirror of ``_WallThermalBoundary`` (solver.py:106-111)."""

    faces: np.ndarray
    condition: str
    value: float
    patch_name: str
    mechanical_condition: str


@dataclass(frozen=True)
class MassFlowOutlet:
    """Mirror of ``_MassFlowOutlet`` (solver.py:99-103)."""

    faces: np.ndarray
    mass_flow: float
    patch_name: str


@dataclass
class Geometry:
    """The subset of the reference ``_Geometry`` that the hot path reads."""

    centers: np.ndarray
    areas: np.ndarray
    inverse_areas: np.ndarray
    face_centers: np.ndarray
    face_normals: np.ndarray
    face_lengths: np.ndarray
    wall_velocities: np.ndarray
    owners: np.ndarray
    neighbours: np.ndarray
    patch_ids: np.ndarray
    patch_kinds: dict
    interior_faces: np.ndarray
    interior_owners: np.ndarray
    interior_neighbours: np.ndarray
    interior_normals: np.ndarray
    interior_lengths: np.ndarray
    interior_owner_offsets: np.ndarray
    interior_neighbour_offsets: np.ndarray
    wall_faces: np.ndarray
    symmetry_faces: np.ndarray
    periodic_faces_a: np.ndarray
    periodic_faces_b: np.ndarray
    velocity_inlet_faces: np.ndarray
    velocity_inlet_states: np.ndarray
    pressure_outlet_faces: np.ndarray
    pressure_outlet_pressures: np.ndarray
    far_field_faces: np.ndarray
    far_field_states: np.ndarray
    pressure_inlets: tuple
    mass_flow_inlets: tuple
    mass_flow_outlets: tuple
    gradient_sources: np.ndarray
    gradient_neighbours: np.ndarray
    gradient_dx: np.ndarray
    gradient_dy: np.ndarray
    gradient_coefficients_x: np.ndarray
    gradient_coefficients_y: np.ndarray
    limiter_cells: np.ndarray
    limiter_dx: np.ndarray
    limiter_dy: np.ndarray
    parabolic_sources: np.ndarray = field(default_factory=lambda: np.empty(0, dtype=np.int64))
    parabolic_neighbours: np.ndarray = field(default_factory=lambda: np.empty(0, dtype=np.int64))
    parabolic_dx: np.ndarray = field(default_factory=lambda: np.empty(0))
    parabolic_dy: np.ndarray = field(default_factory=lambda: np.empty(0))
    periodic_shifts: np.ndarray = field(default_factory=lambda: np.empty((0, 2)))
    # viscous terms (solver.py:1817-1820, 1886-1922): every non-periodic
    # boundary face in face order, and the walls' thermal / mechanical data
    diffusive_boundary_faces: np.ndarray = field(default_factory=lambda: np.empty(0, dtype=np.int64))
    wall_thermal_boundaries: tuple = ()


# ----------------------------------------------------------------- helpers

def _finite_boundary_value(value, description: str) -> float:
    """Mirror of solver.py:4580-4590."""
    if isinstance(value, bool):
        raise SolverError(f"{description} must be finite.")
    try:
        number = float(value)
    except (OverflowError, TypeError, ValueError) as error:
        raise SolverError(f"{description} must be finite.") from error
    if not math.isfinite(number):
        raise SolverError(f"{description} must be finite.")
    return number


def _positive_boundary_value(value, description: str) -> float:
    """Mirror of solver.py:4593-4597."""
    number = _finite_boundary_value(value, description)
    if number <= 0.0:
        raise SolverError(f"{description} must be positive.")
    return number


def _boundary_flow_direction(x, y, description: str) -> np.ndarray:
    """Mirror of solver.py:4600-4612."""
    direction = np.array(
        (
            _finite_boundary_value(x, f"{description} flow direction X"),
            _finite_boundary_value(y, f"{description} flow direction Y"),
        ),
        dtype=float,
    )
    magnitude = float(np.linalg.norm(direction))
    if not math.isfinite(magnitude) or magnitude <= 1e-12:
        raise SolverError(f"{description} needs a non-zero flow direction.")
    return direction / magnitude


def _cells_csr(mesh: FiniteVolumeMesh):
    cells = mesh.cells
    if hasattr(cells, "offsets"):
        return np.ascontiguousarray(cells.offsets, dtype=np.int64), np.ascontiguousarray(cells.nodes, dtype=np.int64)
    arr = np.asarray(cells) if not isinstance(cells, tuple) else None
    if arr is not None and arr.ndim == 2:
        k = arr.shape[1]
        return np.arange(0, k * len(arr) + 1, k, dtype=np.int64), np.ascontiguousarray(arr.ravel(), dtype=np.int64)
    counts = np.fromiter((len(c) for c in cells), dtype=np.int64, count=len(cells))
    offsets = np.concatenate(([0], np.cumsum(counts))).astype(np.int64)
    nodes = np.fromiter((v for c in cells for v in c), dtype=np.int64, count=int(offsets[-1]))
    return offsets, nodes


def _patch_face_ids(patch) -> np.ndarray:
    return np.asarray(patch.face_ids, dtype=np.int64)


# --------------------------------------------------------- periodic matching

def _edge_sort_order(edges: np.ndarray, axis: int) -> np.ndarray:
    """Stable order by the reference's edge sort key (periodic.py:163-172).

    ``edges`` is (n,2,2) with the two end points of each edge sorted
    lexicographically, as ``_patch_edges`` produces (periodic.py:119-125)."""
    first = edges[:, 0, axis]
    second = edges[:, 1, axis]
    k0 = (first + second) / 2.0
    k1 = np.abs(second - first)
    k2 = np.minimum(first, second)
    k3 = np.maximum(first, second)
    return np.lexsort((k3, k2, k1, k0))


def _sorted_edges(points: np.ndarray, faces: np.ndarray, face_ids: np.ndarray) -> np.ndarray:
    a = points[faces[face_ids, 0]]
    b = points[faces[face_ids, 1]]
    swap = (b[:, 0] < a[:, 0]) | ((b[:, 0] == a[:, 0]) & (b[:, 1] < a[:, 1]))
    lo = np.where(swap[:, None], b, a)
    hi = np.where(swap[:, None], a, b)
    return np.stack((lo, hi), axis=1)


def _bounds(edges: np.ndarray):
    pts = edges.reshape(-1, 2)
    return ((float(pts[:, 0].min()), float(pts[:, 0].max())), (float(pts[:, 1].min()), float(pts[:, 1].max())))


def _same_edges(ea: np.ndarray, eb: np.ndarray, tolerance: float, sort_axis: int) -> bool:
    """periodic.py:149-160 and 175-190, vectorised."""
    oa = ea[_edge_sort_order(ea, sort_axis)]
    ob = eb[_edge_sort_order(eb, sort_axis)]
    direct = np.all(np.abs(oa - ob) <= tolerance, axis=(1, 2))
    reverse = np.all(np.abs(oa - ob[:, ::-1, :]) <= tolerance, axis=(1, 2))
    return bool(np.all(direct | reverse))


def detect_periodic_pair(mesh, patch_a_id: int, patch_b_id: int):
    """Restatement of ``detect_periodic_pair`` (periodic.py:10-67)."""
    if patch_a_id == patch_b_id:
        raise ValueError("Select two different patches.")
    patches = {patch.id: patch for patch in mesh.patches}
    try:
        patch_a = patches[patch_a_id]
        patch_b = patches[patch_b_id]
    except KeyError as error:
        raise ValueError("A selected patch is not present in the mesh.") from error
    points = np.asarray(mesh.points, dtype=np.float64)
    faces = np.asarray(mesh.faces, dtype=np.int64)
    ea = _sorted_edges(points, faces, _patch_face_ids(patch_a))
    eb = _sorted_edges(points, faces, _patch_face_ids(patch_b))
    if len(ea) != len(eb):
        raise ValueError("Patches have different numbers of faces.")
    if not len(ea):
        raise ValueError("Periodic patches must contain at least one face.")
    both = np.concatenate((ea, eb))
    bounds = _bounds(both)
    scale = max(1.0, float(np.abs(both).max()), *(upper - lower for lower, upper in bounds))
    tolerance = scale * 1e-9
    bounds_a, bounds_b = _bounds(ea), _bounds(eb)
    matches = []
    for axis, orthogonal, name in ((0, 1, "x"), (1, 0, "y")):
        if (abs(bounds_a[orthogonal][0] - bounds_b[orthogonal][0]) > tolerance
                or abs(bounds_a[orthogonal][1] - bounds_b[orthogonal][1]) > tolerance):
            continue
        translation = ((bounds_b[axis][0] + bounds_b[axis][1]) - (bounds_a[axis][0] + bounds_a[axis][1])) / 2
        if abs(translation) <= tolerance:
            continue
        shifted = ea.copy()
        shifted[:, :, axis] += translation
        shifted = _resort(shifted)
        if _same_edges(shifted, eb, tolerance, orthogonal):
            matches.append((name, abs(translation)))
    if len(matches) != 1:
        raise ValueError("Patches are not a matching translation in exactly one axis (x or y).")
    axis, pitch = matches[0]
    if not math.isfinite(pitch) or pitch <= 0.0:
        raise ValueError("Periodic pitch must be positive and finite.")
    return axis, pitch


def _resort(edges: np.ndarray) -> np.ndarray:
    a, b = edges[:, 0], edges[:, 1]
    swap = (b[:, 0] < a[:, 0]) | ((b[:, 0] == a[:, 0]) & (b[:, 1] < a[:, 1]))
    return np.stack((np.where(swap[:, None], b, a), np.where(swap[:, None], a, b)), axis=1)


def match_periodic_faces(mesh, patch_a_id: int, patch_b_id: int):
    """Restatement of ``match_periodic_faces`` (periodic.py:70-116)."""
    axis, _ = detect_periodic_pair(mesh, patch_a_id, patch_b_id)
    patches = {patch.id: patch for patch in mesh.patches}
    points = np.asarray(mesh.points, dtype=np.float64)
    faces = np.asarray(mesh.faces, dtype=np.int64)
    ids_a = _patch_face_ids(patches[patch_a_id])
    ids_b = _patch_face_ids(patches[patch_b_id])
    ea = _sorted_edges(points, faces, ids_a)
    eb = _sorted_edges(points, faces, ids_b)
    bounds_a, bounds_b = _bounds(ea), _bounds(eb)
    axis_index = 0 if axis == "x" else 1
    tangent_axis = 1 - axis_index
    translation = ((bounds_b[axis_index][0] + bounds_b[axis_index][1])
                   - (bounds_a[axis_index][0] + bounds_a[axis_index][1])) / 2.0
    shift = (translation, 0.0) if axis == "x" else (0.0, translation)
    both = np.concatenate((ea, eb))
    scale = max(1.0, float(np.abs(both).max()), *(upper - lower for lower, upper in _bounds(both)))
    tolerance = scale * 1e-9
    shifted = ea.copy()
    shifted[:, :, 0] += shift[0]
    shifted[:, :, 1] += shift[1]
    shifted = _resort(shifted)
    order_a = _edge_sort_order(shifted, tangent_axis)
    order_b = _edge_sort_order(eb, tangent_axis)
    if not _same_edges(shifted[order_a], eb[order_b], tolerance, tangent_axis):
        raise ValueError("Periodic patch faces do not have a unique matching.")
    return np.column_stack((ids_a[order_a], ids_b[order_b])), shift


# ------------------------------------------------------------------- builder

def build_geometry(mesh: FiniteVolumeMesh, case, host=None) -> Geometry:
    """Restatement of ``_build_geometry`` (solver.py:1654-2238) for the hot path.

    Covers cell/face geometry, periodic pairing, boundary classification and
    values, least-squares gradient entries and coefficients, and limiter
    entries.  Not covered (out of scope for the inviscid path): wall distances
    (SST/viscous only), prescribed-velocity walls (expression evaluation) and
    SST inlet data.

    ``host`` supplies the cell and face loops (``cell_geometry`` and
    ``face_geometry``, solver.py:1654-1696); the default is this library's
    compiled host helpers.  A CPU-only caller may pass its own
    implementation of the same two functions.
    """
    if host is None:
        from . import _lib

        host = _lib.native()
    lib = host
    offsets, nodes = _cells_csr(mesh)
    n_cells = len(offsets) - 1
    points = np.ascontiguousarray(np.asarray(mesh.points, dtype=np.float64))
    faces = np.ascontiguousarray(np.asarray(mesh.faces, dtype=np.int64).reshape(-1, 2))
    owners = np.ascontiguousarray(np.asarray(mesh.face_owners, dtype=np.int64))
    neighbours = np.ascontiguousarray(np.asarray(mesh.face_neighbours, dtype=np.int64))
    patch_ids = np.asarray(mesh.face_patch_ids, dtype=np.int64)
    n_faces = len(faces)

    centers, areas = lib.cell_geometry(offsets, nodes, points)
    face_centers, face_normals, face_lengths = lib.face_geometry(faces, points, centers, owners)

    interior_faces = np.flatnonzero(neighbours >= 0)
    boundary_faces = np.flatnonzero(neighbours < 0)
    conditions = {c.patch_id: c for c in case.boundary_conditions}

    pairs_by_patch = {}
    mappings = []  # (faces_a, faces_b, shift)
    for pair in case.periodic_pairs:
        try:
            axis, pitch = detect_periodic_pair(mesh, pair.patch_a_id, pair.patch_b_id)
            matched, shift = match_periodic_faces(mesh, pair.patch_a_id, pair.patch_b_id)
        except ValueError as error:
            raise SolverError(f"Invalid periodic boundary pair: {error}") from error
        if pair.axis != axis or not math.isclose(pair.pitch, pitch, rel_tol=1e-9, abs_tol=max(pitch, 1.0) * 1e-9):
            raise SolverError("A periodic pair has a stale axis or pitch.")
        if (pair.patch_a_id not in conditions or pair.patch_b_id not in conditions
                or conditions[pair.patch_a_id].kind != "Periodic"
                or conditions[pair.patch_b_id].kind != "Periodic"):
            raise SolverError("Both patches in every periodic pair must be Periodic.")
        if pair.patch_a_id in pairs_by_patch or pair.patch_b_id in pairs_by_patch:
            raise SolverError("A patch cannot belong to multiple periodic pairs.")
        pairs_by_patch[pair.patch_a_id] = pair
        pairs_by_patch[pair.patch_b_id] = pair
        mappings.append((matched[:, 0], matched[:, 1], shift))

    periodic_patch_ids = {pid for pid, c in conditions.items() if c.kind == "Periodic"}
    if periodic_patch_ids != set(pairs_by_patch):
        raise SolverError("Each Periodic boundary must belong to exactly one pair.")
    if set(conditions) != {patch.id for patch in mesh.patches}:
        raise SolverError("Boundary conditions must be defined for every mesh patch.")
    for pid, condition in conditions.items():
        if condition.kind not in SUPPORTED_KINDS:
            raise SolverError(f"Boundary type '{condition.kind}' is not implemented by the solver.")
        if condition.kind == "Periodic" and pid not in pairs_by_patch:
            raise SolverError(f"Periodic patch '{condition.patch_name}' has no pair.")

    periodic_a = np.concatenate([m[0] for m in mappings]) if mappings else np.empty(0, dtype=np.int64)
    periodic_b = np.concatenate([m[1] for m in mappings]) if mappings else np.empty(0, dtype=np.int64)
    shifts = (np.concatenate([np.tile(np.asarray(m[2], dtype=float), (len(m[0]), 1)) for m in mappings])
              if mappings else np.empty((0, 2)))
    is_periodic_face = np.zeros(n_faces, dtype=bool)
    is_periodic_face[periodic_a] = True
    is_periodic_face[periodic_b] = True
    if np.any(is_periodic_face & (neighbours >= 0)):
        raise SolverError("Periodic pairs must reference boundary faces.")
    kind_of_patch = {pid: c.kind for pid, c in conditions.items()}
    boundary_kinds = np.array([kind_of_patch.get(int(p), "") for p in patch_ids[boundary_faces]], dtype=object) \
        if len(boundary_faces) < 200000 else None
    if boundary_kinds is None:
        lookup = {pid: i for i, pid in enumerate(kind_of_patch)}
        codes = np.array([lookup.get(int(p), -1) for p in np.unique(patch_ids[boundary_faces])])
        del codes
        boundary_kinds = np.array([kind_of_patch.get(int(p), "") for p in patch_ids[boundary_faces]], dtype=object)
    periodic_patch_face = np.array([k == "Periodic" for k in boundary_kinds], dtype=bool)
    if np.any(periodic_patch_face & ~is_periodic_face[boundary_faces]):
        raise SolverError("Periodic patches contain unmatched faces.")
    not_periodic = ~is_periodic_face[boundary_faces]
    wall_mask = not_periodic & np.isin(boundary_kinds, ("Wall", "Symmetry"))
    wall_faces = boundary_faces[wall_mask]
    symmetry_faces = boundary_faces[not_periodic & (boundary_kinds == "Symmetry")]

    gas_constant = case.numerics.gas_constant
    vin_faces, vin_states = [], []
    pout_faces, pout_pressures = [], []
    far_faces, far_states = [], []
    pressure_inlets, mass_flow_inlets, mass_flow_outlets = [], [], []
    wall_thermal = []
    boundary_patch = patch_ids[boundary_faces]
    for pid, condition in conditions.items():
        fids = boundary_faces[boundary_patch == pid]
        name = condition.patch_name
        if condition.kind == "Velocity Inlet":
            density = _positive_boundary_value(condition.values.get("density", 1.225), f"Density for velocity inlet '{name}'")
            temperature = _positive_boundary_value(condition.values.get("temperature", 288.15), f"Temperature for velocity inlet '{name}'")
            vx = _finite_boundary_value(condition.values.get("velocity_x", 0.0), f"Velocity X for inlet '{name}'")
            vy = _finite_boundary_value(condition.values.get("velocity_y", 0.0), f"Velocity Y for inlet '{name}'")
            pressure = density * gas_constant * temperature
            if not math.isfinite(pressure) or pressure <= 0.0:
                raise SolverError(f"Velocity inlet '{name}' produces invalid pressure.")
            vin_faces.append(fids)
            vin_states.append(np.tile((density, vx, vy, pressure), (len(fids), 1)))
        elif condition.kind == "Wall":
            if condition.mechanical_condition == "Prescribed velocity":
                raise SolverError("Prescribed-velocity walls need the reference geometry (expression evaluation).")
            if case.numerics.viscosity_model != "Inviscid":
                mechanical = condition.mechanical_condition
                if mechanical not in ("Slip", "No-slip", "Prescribed velocity"):
                    raise SolverError(f"Unsupported mechanical condition on wall '{name}'.")
                thermal = condition.thermal_condition
                if thermal == "Temperature":
                    value = _positive_boundary_value(condition.values.get("temperature", 300.0),
                                                     f"Wall temperature for '{name}'")
                elif thermal == "Heat Flux":
                    value = _finite_boundary_value(condition.values.get("heat_flux", 0.0),
                                                   f"Wall heat flux for '{name}'")
                else:
                    raise SolverError(f"Unsupported thermal condition on wall '{name}'.")
                wall_thermal.append(WallThermalBoundary(fids, thermal, value, name, mechanical))
        elif condition.kind == "Pressure Outlet":
            pressure = _positive_boundary_value(condition.values.get("pressure", 101325.0), f"Static pressure for outlet '{name}'")
            pout_faces.append(fids)
            pout_pressures.append(np.full(len(fids), pressure))
        elif condition.kind == "Pressure Inlet":
            total_pressure = _positive_boundary_value(condition.values.get("pressure", 101325.0), f"Total pressure for inlet '{name}'")
            total_temperature = _positive_boundary_value(condition.values.get("temperature", 288.15), f"Total temperature for inlet '{name}'")
            direction = _boundary_flow_direction(condition.values.get("velocity_x", 1.0), condition.values.get("velocity_y", 0.0), f"Pressure inlet '{name}'")
            pressure_inlets.append(PressureInlet(fids, total_pressure, total_temperature, direction, name))
        elif condition.kind == "Mass Flow Inlet":
            mass_flow = _positive_boundary_value(condition.values.get("mass_flow", 1.0), f"Mass flow for inlet '{name}'")
            total_temperature = _positive_boundary_value(condition.values.get("temperature", 288.15), f"Total temperature for inlet '{name}'")
            direction = _boundary_flow_direction(condition.values.get("velocity_x", 1.0), condition.values.get("velocity_y", 0.0), f"Mass-flow inlet '{name}'")
            mass_flow_inlets.append(MassFlowInlet(fids, mass_flow, total_temperature, direction, name))
        elif condition.kind == "Mass Flow Outlet":
            mass_flow = _positive_boundary_value(condition.values.get("mass_flow", 1.0), f"Mass flow for outlet '{name}'")
            mass_flow_outlets.append(MassFlowOutlet(fids, mass_flow, name))
        elif condition.kind == "Far Field":
            density = _positive_boundary_value(condition.values.get("density", 1.225), f"Density for far field '{name}'")
            vx = _finite_boundary_value(condition.values.get("velocity_x", 0.0), f"Velocity X for far field '{name}'")
            vy = _finite_boundary_value(condition.values.get("velocity_y", 0.0), f"Velocity Y for far field '{name}'")
            pressure = _positive_boundary_value(condition.values.get("pressure", 101325.0), f"Pressure for far field '{name}'")
            far_faces.append(fids)
            far_states.append(np.tile((density, vx, vy, pressure), (len(fids), 1)))

    def cat_int(parts):
        return np.concatenate(parts).astype(np.int64) if parts else np.empty(0, dtype=np.int64)

    def cat_state(parts, width):
        return np.concatenate(parts).reshape(-1, width) if parts else np.empty((0, width))

    # Least-squares gradient entries (solver.py:2004-2021): per interior face the
    # owner entry then the neighbour entry, then per periodic pair.
    io = owners[interior_faces]
    ineigh = neighbours[interior_faces]
    pa_own = owners[periodic_a]
    pb_own = owners[periodic_b]
    src = np.concatenate((np.column_stack((io, ineigh)).ravel(), np.column_stack((pa_own, pb_own)).ravel()))
    nbr = np.concatenate((np.column_stack((ineigh, io)).ravel(), np.column_stack((pb_own, pa_own)).ravel()))
    src = src.astype(np.int64)
    nbr = nbr.astype(np.int64)
    lim_cells = np.concatenate((owners, ineigh))
    device_numeric = getattr(lib, "gradient_and_limiter_offsets", None)
    if device_numeric is not None:
        # the offsets, weights, moment sums, coefficients and limiter offsets
        # below, computed by the library's kernels in the same order
        gdx, gdy, cx, cy, lim_dx, lim_dy = device_numeric(
            n_cells, src, nbr, 2 * len(interior_faces), shifts, centers, face_centers,
            np.concatenate((np.arange(n_faces, dtype=np.int64), interior_faces)), lim_cells)
    else:
        delta = centers[ineigh] - centers[io]
        pdelta = (centers[pb_own] - shifts) - centers[pa_own]
        gdx = np.concatenate((np.column_stack((delta[:, 0], -delta[:, 0])).ravel(),
                              np.column_stack((pdelta[:, 0], -pdelta[:, 0])).ravel()))
        gdy = np.concatenate((np.column_stack((delta[:, 1], -delta[:, 1])).ravel(),
                              np.column_stack((pdelta[:, 1], -pdelta[:, 1])).ravel()))

        # Least-squares coefficients (solver.py:2050-2078).
        dist2 = gdx * gdx + gdy * gdy
        weights = 1.0 / np.maximum(dist2, 1e-300)
        wdx = weights * gdx
        wdy = weights * gdy
        mxx = np.zeros(n_cells)
        mxy = np.zeros(n_cells)
        myy = np.zeros(n_cells)
        np.add.at(mxx, src, wdx * gdx)
        np.add.at(mxy, src, wdx * gdy)
        np.add.at(myy, src, wdy * gdy)
        det = mxx * myy - mxy * mxy
        valid = det > 1e-14 * np.maximum(mxx * myy, 1e-300)
        ixx = np.zeros(n_cells)
        ixy = np.zeros(n_cells)
        iyy = np.zeros(n_cells)
        ixx[valid] = myy[valid] / det[valid]
        ixy[valid] = -mxy[valid] / det[valid]
        iyy[valid] = mxx[valid] / det[valid]
        cx = ixx[src] * wdx + ixy[src] * wdy
        cy = ixy[src] * wdx + iyy[src] * wdy

        # Limiter entries (solver.py:2098-2105): every face's owner, then every
        # interior face's neighbour.
        lim_dx = np.concatenate((face_centers[:, 0] - centers[owners, 0],
                                 face_centers[interior_faces, 0] - centers[ineigh, 0]))
        lim_dy = np.concatenate((face_centers[:, 1] - centers[owners, 1],
                                 face_centers[interior_faces, 1] - centers[ineigh, 1]))

    parabolic = (np.empty(0, dtype=np.int64), np.empty(0, dtype=np.int64), np.empty(0), np.empty(0))
    if case.numerics.reconstruction == "MUSCL parabolic":
        domain_scale = max(float(points[:, 0].max() - points[:, 0].min()), float(points[:, 1].max() - points[:, 1].min()), 1e-12)
        search = getattr(lib, "parabolic_stencil", None) or parabolic_stencil
        parabolic = search(n_cells, src, nbr, gdx, gdy, domain_scale)

    return Geometry(
        centers=centers,
        areas=areas,
        inverse_areas=1.0 / areas,
        face_centers=face_centers,
        face_normals=face_normals,
        face_lengths=face_lengths,
        wall_velocities=np.zeros((n_faces, 2)),
        owners=owners,
        neighbours=neighbours,
        patch_ids=patch_ids,
        patch_kinds=dict(kind_of_patch),
        interior_faces=interior_faces,
        interior_owners=io,
        interior_neighbours=ineigh,
        interior_normals=face_normals[interior_faces],
        interior_lengths=face_lengths[interior_faces],
        interior_owner_offsets=face_centers[interior_faces] - centers[io],
        interior_neighbour_offsets=face_centers[interior_faces] - centers[ineigh],
        wall_faces=wall_faces.astype(np.int64),
        symmetry_faces=symmetry_faces.astype(np.int64),
        periodic_faces_a=periodic_a.astype(np.int64),
        periodic_faces_b=periodic_b.astype(np.int64),
        velocity_inlet_faces=cat_int(vin_faces),
        velocity_inlet_states=cat_state(vin_states, 4),
        pressure_outlet_faces=cat_int(pout_faces),
        pressure_outlet_pressures=np.concatenate(pout_pressures) if pout_pressures else np.empty(0),
        far_field_faces=cat_int(far_faces),
        far_field_states=cat_state(far_states, 4),
        pressure_inlets=tuple(pressure_inlets),
        mass_flow_inlets=tuple(mass_flow_inlets),
        mass_flow_outlets=tuple(mass_flow_outlets),
        gradient_sources=src,
        gradient_neighbours=nbr,
        gradient_dx=gdx,
        gradient_dy=gdy,
        gradient_coefficients_x=cx,
        gradient_coefficients_y=cy,
        limiter_cells=lim_cells.astype(np.int64),
        limiter_dx=lim_dx,
        limiter_dy=lim_dy,
        parabolic_sources=parabolic[0],
        parabolic_neighbours=parabolic[1],
        parabolic_dx=parabolic[2],
        parabolic_dy=parabolic[3],
        periodic_shifts=shifts,
        diffusive_boundary_faces=boundary_faces[not_periodic].astype(np.int64),
        wall_thermal_boundaries=tuple(wall_thermal),
    )


def parabolic_stencil(cell_count, sources, neighbours, dx, dy, domain_scale):
    """Two-ring stencil by breadth-first search, restating ``_parabolic_stencil``
    (solver.py:2241-2291): same visiting order, same duplicate key (neighbour id
    plus the offset rounded to 10 decimals of the domain scale)."""
    order = np.argsort(sources, kind="stable")
    starts = np.searchsorted(sources[order], np.arange(cell_count + 1))
    adj_n = neighbours[order]
    adj_x = dx[order]
    adj_y = dy[order]
    out_s, out_n, out_x, out_y = [], [], [], []
    for source in range(cell_count):
        frontier = [(source, 0.0, 0.0)]
        seen = {(source, 0, 0)}
        for _depth in range(2):
            next_frontier = []
            for current, ox, oy in frontier:
                for k in range(starts[current], starts[current + 1]):
                    nb = int(adj_n[k])
                    px = ox + float(adj_x[k])
                    py = oy + float(adj_y[k])
                    key = (nb, round(px / domain_scale, 10), round(py / domain_scale, 10))
                    if key in seen:
                        continue
                    seen.add(key)
                    next_frontier.append((nb, px, py))
                    if math.hypot(px, py) > domain_scale * 1e-12:
                        out_s.append(source)
                        out_n.append(nb)
                        out_x.append(px)
                        out_y.append(py)
            frontier = next_frontier
    return (np.asarray(out_s, dtype=np.int64), np.asarray(out_n, dtype=np.int64),
            np.asarray(out_x, dtype=float), np.asarray(out_y, dtype=float))
