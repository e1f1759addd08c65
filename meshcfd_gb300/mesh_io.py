"""Reader for MeshCAD's versioned finite-volume mesh JSON format, the on-disk
format the residual path's geometry comes from.

Mirrors the reference reader (io/mesh_io.py): ``FORMAT_NAME``,
``FORMAT_VERSION``, ``MeshImportError``, ``mesh_from_dict`` (mesh_io.py:133),
``load_mesh`` (mesh_io.py:448) and ``mesh_to_dict`` (mesh_io.py:460), with the
same checks in the same order and the same messages, so a file the reference
rejects is rejected here with the reference's message.  The reference checks
every node, face and cell in Python loops; here each section is checked on
NumPy arrays first, and only a section that fails is re-checked element by
element to report the reference's first error.  The mesh comes back with
array fields (``model.FiniteVolumeMesh``): points (N, 2) float64, faces
(F, 2) and face_owners / face_neighbours / face_patch_ids (F,) int64, cells as
a vertex CSR (``meshes.CellArray``) in the reference's loop order, and the
cell face lists and signs as CSRs (``CellArray`` whose ``nodes`` are face ids
resp. signs) -- the form ``geometry.build_geometry`` takes directly.
"""

from __future__ import annotations

import json
import math
from pathlib import Path
from typing import Any

import numpy as np

from .meshes import CellArray
from .model import BoundaryCurve, FiniteVolumeMesh, MeshPatch, RefinementRecord

FORMAT_NAME = "meshcad-mesh"
FORMAT_VERSION = 1
NO_NEIGHBOUR = -1

_I64_MIN, _I64_MAX = np.iinfo(np.int64).min, np.iinfo(np.int64).max


class MeshImportError(ValueError):
    """Raised when a mesh file is unsupported or invalid."""


# ------------------------------------------------------------ scalar checks
# The reference's element checks (mesh_io.py:26-48), used where a section
# fails its array check and the first offending element must be reported.

def _integer(value: Any, description: str) -> int:
    if isinstance(value, bool) or not isinstance(value, int):
        raise MeshImportError(f"{description} must be an integer.")
    return value


def _finite_number(value: Any, description: str) -> float:
    if isinstance(value, bool):
        raise MeshImportError(f"{description} must be a finite number.")
    try:
        number = float(value)
    except (OverflowError, TypeError, ValueError) as error:
        raise MeshImportError(f"{description} must be a finite number.") from error
    if not math.isfinite(number):
        raise MeshImportError(f"{description} must be a finite number.")
    return number


def _clipped_int64(values: list) -> np.ndarray:
    """Python ints as int64; values beyond int64 are clipped (they fail every
    range check here exactly as the unbounded values fail the reference's)."""
    try:
        return np.array(values, dtype=np.int64)
    except OverflowError:
        return np.array([min(max(v, _I64_MIN), _I64_MAX) for v in values], dtype=np.int64)


def _integer_array(value: Any, description: str) -> np.ndarray:
    """The reference's ``_integer_list`` (mesh_io.py:32-35) as an int64 array."""
    if not isinstance(value, list):
        raise MeshImportError(f"{description} must be a list.")
    if value and {type(item) for item in value} != {int}:
        for item in value:
            _integer(item, description)
    return _clipped_int64(value)


def _is_pair_list(rows: list) -> bool:
    return all(isinstance(row, list) and len(row) == 2 for row in rows)


# ---------------------------------------------------------- boundary curves

def _spline_point(points, parameter: float) -> tuple:
    """Catmull-Rom spline through the control points, end controls repeated
    (core/curves.py:8-38)."""
    if len(points) == 2:
        return tuple(points[0][axis] + (points[1][axis] - points[0][axis]) * parameter for axis in (0, 1))
    segments = len(points) - 1
    scaled = parameter * segments
    index = min(int(scaled), segments - 1)
    local = scaled - index
    local2 = local * local
    local3 = local2 * local
    p0, p1, p2, p3 = (points[max(0, index - 1)], points[index], points[index + 1],
                      points[min(index + 2, len(points) - 1)])
    out = []
    for axis in (0, 1):
        a, b, c, d = p0[axis], p1[axis], p2[axis], p3[axis]
        out.append(0.5 * (2.0 * b + (-a + c) * local + (2.0 * a - 5.0 * b + 4.0 * c - d) * local2
                          + (-a + 3.0 * b - 3.0 * c + d) * local3))
    return out[0], out[1]


def evaluate_boundary_curve(geometry: dict, parameter: float) -> tuple:
    """A MeshCAD boundary-curve descriptor at its normalised parameter
    (core/curves.py:41-80): line, circular arc (counter-clockwise from the
    start angle), spline, or a spline segment with end offsets."""
    parameter = max(0.0, min(1.0, parameter))
    kind = geometry.get("type")
    if kind == "line":
        start, end = geometry["start"], geometry["end"]
        return tuple(start[axis] + (end[axis] - start[axis]) * parameter for axis in (0, 1))
    if kind == "arc":
        center = geometry["center"]
        span = geometry["end_angle"] - geometry["start_angle"]
        while span <= 0.0:
            span += 2.0 * math.pi
        angle = geometry["start_angle"] + span * parameter
        return center[0] + geometry["radius"] * math.cos(angle), center[1] + geometry["radius"] * math.sin(angle)
    if kind in ("spline", "spline_segment"):
        points = geometry["points"]
        if kind == "spline":
            return _spline_point(points, parameter)
        start_t, end_t = geometry["start_t"], geometry["end_t"]
        point = _spline_point(points, start_t + (end_t - start_t) * parameter)
        start_offset = geometry.get("start_offset", (0.0, 0.0))
        end_offset = geometry.get("end_offset", (0.0, 0.0))
        return tuple(point[axis] + start_offset[axis] * (1.0 - parameter) + end_offset[axis] * parameter
                     for axis in (0, 1))
    raise ValueError(f"Unsupported boundary curve type: {kind!r}.")


def _curve_geometry(value: Any, description: str) -> dict:
    """Validated copy of a curve descriptor (mesh_io.py:51-130)."""
    if not isinstance(value, dict):
        raise MeshImportError(f"{description} must be an object.")
    kind = value.get("type")
    if kind == "line":
        keys = ("start", "end")
    elif kind == "arc":
        center = value.get("center")
        if not isinstance(center, list) or len(center) != 2:
            raise MeshImportError(f"{description} has an invalid arc center.")
        radius = _finite_number(value.get("radius"), f"{description} arc radius")
        if radius <= 0.0:
            raise MeshImportError(f"{description} arc radius must be positive.")
        return {
            "type": kind,
            "center": [_finite_number(item, f"{description} arc center") for item in center],
            "radius": radius,
            "start_angle": _finite_number(value.get("start_angle"), f"{description} arc start angle"),
            "end_angle": _finite_number(value.get("end_angle"), f"{description} arc end angle"),
        }
    elif kind in ("spline", "spline_segment"):
        raw = value.get("points")
        if not isinstance(raw, list) or len(raw) < 2 or not _is_pair_list(raw):
            raise MeshImportError(f"{description} has invalid spline points.")
        points = [[_finite_number(item, f"{description} spline point") for item in point] for point in raw]
        if kind == "spline":
            return {"type": kind, "points": points}
        start_t = _finite_number(value.get("start_t"), f"{description} spline start parameter")
        end_t = _finite_number(value.get("end_t"), f"{description} spline end parameter")
        if not 0.0 <= start_t < end_t <= 1.0:
            raise MeshImportError(f"{description} has invalid spline parameters.")
        offsets = {}
        for key in ("start_offset", "end_offset"):
            offset = value.get(key, [0.0, 0.0])
            if not isinstance(offset, list) or len(offset) != 2:
                raise MeshImportError(f"{description} has an invalid {key}.")
            offsets[key] = [_finite_number(item, f"{description} {key}") for item in offset]
        return {"type": kind, "points": points, "start_t": start_t, "end_t": end_t, **offsets}
    else:
        raise MeshImportError(f"{description} has an unsupported geometry type.")
    coordinates = {}
    for key in keys:
        point = value.get(key)
        if not isinstance(point, list) or len(point) != 2:
            raise MeshImportError(f"{description} has invalid {key} coordinates.")
        coordinates[key] = [_finite_number(item, f"{description} {key} coordinate") for item in point]
    return {"type": kind, **coordinates}


# ------------------------------------------------------------------ sections

def _parse_points(coordinates: list) -> np.ndarray:
    if _is_pair_list(coordinates) and {type(v) for row in coordinates for v in row} <= {int, float}:
        try:
            points = np.array(coordinates, dtype=np.float64)
        except OverflowError:
            points = None
        if points is not None and np.isfinite(points).all():
            return points
    # element by element, as the reference (mesh_io.py:153-164)
    out = []
    for index, coordinate in enumerate(coordinates):
        if not isinstance(coordinate, list) or len(coordinate) != 2:
            raise MeshImportError(f"Node {index} must have two coordinates.")
        try:
            point = (float(coordinate[0]), float(coordinate[1]))
        except (TypeError, ValueError) as error:
            raise MeshImportError(f"Node {index} has invalid coordinates.") from error
        if not all(math.isfinite(value) for value in point):
            raise MeshImportError(f"Node {index} coordinates must be finite.")
        out.append(point)
    return np.array(out, dtype=np.float64)


def _parse_faces(face_nodes: list, n_points: int) -> np.ndarray:
    if _is_pair_list(face_nodes) and {type(v) for row in face_nodes for v in row} == {int}:
        faces = _clipped_int64(face_nodes)
        bad = (faces[:, 0] == faces[:, 1]) | (faces < 0).any(axis=1) | (faces >= n_points).any(axis=1)
        if not bad.any():
            return faces
    for face_id, nodes in enumerate(face_nodes):  # mesh_io.py:168-178
        if not isinstance(nodes, list) or len(nodes) != 2:
            raise MeshImportError(f"Face {face_id} must have exactly two nodes.")
        node_ids = tuple(_integer(node, f"Face {face_id} node") for node in nodes)
        if node_ids[0] == node_ids[1] or any(node < 0 or node >= n_points for node in node_ids):
            raise MeshImportError(f"Face {face_id} references invalid nodes.")
    raise AssertionError("unreachable: the array check failed but no face is invalid")


def _parse_patches(raw_patches: list, n_faces: int) -> list:
    if not isinstance(raw_patches, list):
        raise MeshImportError("Patches must be a list.")
    patches, ids, names = [], set(), set()
    for item in raw_patches:  # mesh_io.py:189-205
        if not isinstance(item, dict):
            raise MeshImportError("Each patch must be a JSON object.")
        patch_id = _integer(item.get("id"), "Patch identifier")
        name = item.get("name")
        if not isinstance(name, str) or not name.strip():
            raise MeshImportError(f"Patch {patch_id} must have a non-empty name.")
        if patch_id in ids or name in names:
            raise MeshImportError("Patch identifiers and names must be unique.")
        face_ids = _integer_array(item.get("faces"), f"Patch {name} faces")
        if ((face_ids < 0) | (face_ids >= n_faces)).any():
            raise MeshImportError(f"Patch {name} references invalid faces.")
        patches.append(MeshPatch(patch_id, name, face_ids))
        ids.add(patch_id)
        names.add(name)
    return patches


def _check_face_links(owners, neighbours, patch_of_face, n_cells: int, patch_ids: set) -> None:
    """mesh_io.py:212-227."""
    known = np.array(sorted(patch_ids), dtype=np.int64)
    if ((patch_of_face != NO_NEIGHBOUR) & ~np.isin(patch_of_face, known)).any():
        raise MeshImportError("A face references an unknown boundary patch.")
    boundary = neighbours == NO_NEIGHBOUR
    bad = (owners < 0) | (owners >= n_cells)
    bad |= ~boundary & ((neighbours < 0) | (neighbours >= n_cells) | (neighbours == owners))
    bad |= boundary != (patch_of_face != NO_NEIGHBOUR)
    if bad.any():
        face_id = int(np.argmax(bad))
        owner, neighbour, patch_id = int(owners[face_id]), int(neighbours[face_id]), int(patch_of_face[face_id])
        if owner < 0 or owner >= n_cells:
            raise MeshImportError(f"Face {face_id} references an invalid owner cell.")
        if neighbour != NO_NEIGHBOUR and (neighbour < 0 or neighbour >= n_cells or neighbour == owner):
            raise MeshImportError(f"Face {face_id} references an invalid neighbour cell.")
        raise MeshImportError(f"Face {face_id} has inconsistent boundary data.")


def _parse_curves(raw_curves: Any, faces: np.ndarray, points: np.ndarray, neighbours, patch_of_face) -> tuple:
    """mesh_io.py:229-299."""
    if not isinstance(raw_curves, list) or len(raw_curves) != len(faces):
        raise MeshImportError("Boundary curves must contain one entry per face.")
    parsed = []
    for face_id, raw in enumerate(raw_curves):
        if raw is None:
            parsed.append(None)
            continue
        if not isinstance(raw, dict):
            raise MeshImportError(f"Boundary curve {face_id} must be an object.")
        if neighbours[face_id] != NO_NEIGHBOUR:
            raise MeshImportError(f"Internal face {face_id} cannot have a boundary curve.")
        patch_id = _integer(raw.get("patch_id"), f"Boundary curve {face_id} patch")
        if patch_id != patch_of_face[face_id]:
            raise MeshImportError(f"Boundary curve {face_id} has an inconsistent patch.")
        raw_parameters = raw.get("parameters")
        if not isinstance(raw_parameters, list) or len(raw_parameters) != 2:
            raise MeshImportError(f"Boundary curve {face_id} must have two parameters.")
        start, end = (_finite_number(item, f"Boundary curve {face_id} parameter") for item in raw_parameters)
        if not (0.0 <= start <= 1.0 and 0.0 <= end <= 1.0 and start != end):
            raise MeshImportError(f"Boundary curve {face_id} has invalid parameters.")
        geometry = _curve_geometry(raw.get("geometry"), f"Boundary curve {face_id}")
        curve = BoundaryCurve(geometry, start, end, patch_id)
        nodes = (int(faces[face_id, 0]), int(faces[face_id, 1]))
        scale = max(1.0, *(abs(float(v)) for node in nodes for v in points[node]))
        tolerance = scale * 1.0e-8
        for node_id, parameter in zip(nodes, (start, end)):
            try:
                evaluated = evaluate_boundary_curve(geometry, parameter)
            except (ArithmeticError, KeyError, TypeError, ValueError) as error:
                raise MeshImportError(f"Boundary curve {face_id} cannot be evaluated.") from error
            if any(abs(evaluated[axis] - float(points[node_id, axis])) > tolerance for axis in (0, 1)):
                raise MeshImportError(f"Boundary curve {face_id} does not match its face nodes.")
        parsed.append(curve)
    return tuple(parsed)


def _cells_csr(cell_faces: list, cell_signs: list):
    """Face ids and signs of every cell as CSRs, when every entry is a list
    of plain ints; None otherwise."""
    if not all(isinstance(ids, list) for ids in cell_faces) or not all(isinstance(s, list) for s in cell_signs):
        return None
    counts = np.fromiter((len(ids) for ids in cell_faces), dtype=np.int64, count=len(cell_faces))
    sign_counts = np.fromiter((len(s) for s in cell_signs), dtype=np.int64, count=len(cell_signs))
    if not np.array_equal(counts, sign_counts) or (counts < 3).any():
        return None
    flat_ids = [f for ids in cell_faces for f in ids]
    flat_signs = [v for s in cell_signs for v in s]
    if {type(v) for v in flat_ids} != {int} or {type(v) for v in flat_signs} != {int}:
        return None
    offsets = np.zeros(len(cell_faces) + 1, dtype=np.int64)
    np.cumsum(counts, out=offsets[1:])
    return offsets, _clipped_int64(flat_ids), _clipped_int64(flat_signs)


def _order_loop(edges: list):
    """The reference's node-loop construction for one cell (mesh_io.py:323-348):
    from the first directed edge, repeatedly the first remaining edge that
    starts where the last one ends.  Returns the loop's nodes, or None."""
    edges = list(edges)
    ordered = [edges.pop(0)]
    while edges:
        start = ordered[-1][1]
        nxt = next((i for i, edge in enumerate(edges) if edge[0] == start), None)
        if nxt is None:
            break
        ordered.append(edges.pop(nxt))
    if edges or ordered[-1][1] != ordered[0][0]:
        return None
    return [edge[0] for edge in ordered]


def _cell_loops(offsets, face_ids, signs, faces: np.ndarray):
    """Vertex loops of all cells.  Returns (nodes in loop order, per-cell ok).
    Cells whose directed edges start at distinct nodes follow the unique
    successor of each edge on arrays; the others take the reference's
    first-match loop."""
    n_cells = len(offsets) - 1
    counts = np.diff(offsets)
    cell_of = np.repeat(np.arange(n_cells, dtype=np.int64), counts)
    fwd = signs == 1
    start = np.where(fwd, faces[face_ids, 0], faces[face_ids, 1])
    end = np.where(fwd, faces[face_ids, 1], faces[face_ids, 0])
    n_nodes = int(faces.max()) + 1
    key = cell_of * n_nodes + start
    order = np.argsort(key, kind="stable")
    sorted_key = key[order]
    dup = np.zeros(len(key), dtype=bool)
    dup[order[1:]] = sorted_key[1:] == sorted_key[:-1]
    dup[order[:-1]] |= sorted_key[1:] == sorted_key[:-1]
    ambiguous = np.zeros(n_cells, dtype=bool)
    np.logical_or.at(ambiguous, cell_of, dup)
    # successor of each entry: the entry of the same cell starting at its end
    want = cell_of * n_nodes + end
    pos = np.searchsorted(sorted_key, want)
    pos_c = np.minimum(pos, len(sorted_key) - 1)
    found = sorted_key[pos_c] == want
    succ = np.where(found, order[pos_c], -1)
    # follow the successors from each cell's first entry
    loop = np.arange(len(key), dtype=np.int64)  # entry at each position of the cell's loop
    ok = ~ambiguous
    visited = np.zeros(len(key), dtype=bool)
    current = offsets[:-1].copy()
    loop[offsets[:-1]] = current
    visited[current] = True
    for t in range(1, int(counts.max()) if n_cells else 0):
        active = np.nonzero(ok & (counts > t))[0]
        if not len(active):
            break
        nxt = succ[current[active]]
        good = nxt >= 0
        good[good] &= ~visited[nxt[good]]
        ok[active[~good]] = False
        active, nxt = active[good], nxt[good]
        visited[nxt] = True
        current[active] = nxt
        loop[offsets[active] + t] = nxt
    last_end = end[current]
    ok &= last_end == start[offsets[:-1]]
    nodes = start[loop]
    for c in np.nonzero(ambiguous)[0]:
        a, b = offsets[c], offsets[c + 1]
        loop_nodes = _order_loop(list(zip(start[a:b].tolist(), end[a:b].tolist())))
        if loop_nodes is not None:
            nodes[a:b] = loop_nodes
            ok[c] = True
    return nodes, ok


def _check_cells_one_by_one(cell_faces, cell_signs, faces: np.ndarray) -> None:
    """mesh_io.py:311-349, element by element: raises the first cell error."""
    n_faces = len(faces)
    for cell_id, (raw_face_ids, raw_signs) in enumerate(zip(cell_faces, cell_signs)):
        ids = [int(v) for v in _integer_array(raw_face_ids, f"Cell {cell_id} faces")]
        signs = [int(v) for v in _integer_array(raw_signs, f"Cell {cell_id} face signs")]
        if len(ids) < 3 or len(ids) != len(signs):
            raise MeshImportError(f"Cell {cell_id} must have at least three faces.")
        if any(face < 0 or face >= n_faces for face in ids):
            raise MeshImportError(f"Cell {cell_id} references invalid faces.")
        if any(sign not in (-1, 1) for sign in signs):
            raise MeshImportError(f"Cell {cell_id} face signs must be -1 or 1.")
        edges = [(int(faces[f, 0]), int(faces[f, 1])) if s == 1 else (int(faces[f, 1]), int(faces[f, 0]))
                 for f, s in zip(ids, signs)]
        if _order_loop(edges) is None:
            raise MeshImportError(f"Cell {cell_id} faces do not form a closed node loop.")


def _parse_cells(cell_faces: list, cell_signs: list, faces: np.ndarray):
    csr = _cells_csr(cell_faces, cell_signs)
    if csr is not None:
        offsets, face_ids, signs = csr
        if not (((face_ids < 0) | (face_ids >= len(faces))).any() or ((signs != 1) & (signs != -1)).any()):
            nodes, ok = _cell_loops(offsets, face_ids, signs, faces)
            if ok.all():
                return CellArray(offsets, nodes), CellArray(offsets, face_ids), CellArray(offsets, signs)
    _check_cells_one_by_one(cell_faces, cell_signs, faces)
    raise AssertionError("unreachable: the array check failed but no cell is invalid")


def _check_patch_membership(patches: list, patch_of_face: np.ndarray) -> None:
    """mesh_io.py:351-363."""
    for patch in patches:
        if (patch_of_face[patch.face_ids] != patch.id).any():
            raise MeshImportError(f"Patch {patch.name} contains an unrelated face.")
    listed = np.concatenate([p.face_ids for p in patches]) if patches else np.zeros(0, dtype=np.int64)
    if len(np.unique(listed)) != len(listed):
        raise MeshImportError("A boundary face cannot belong to multiple patches.")
    member = np.zeros(len(patch_of_face), dtype=bool)
    member[listed] = True
    bad = (patch_of_face != NO_NEIGHBOUR) != member
    if bad.any():
        raise MeshImportError(f"Face {int(np.argmax(bad))} has inconsistent patch membership.")


def _parse_refinement(raw: Any, n_cells: int):
    """mesh_io.py:365-427."""
    if not isinstance(raw, dict):
        raise MeshImportError("Refinement metadata must be an object.")
    raw_cell_ids = raw.get("cell_ids", [])
    raw_cell_levels = raw.get("cell_levels", [])
    if not isinstance(raw_cell_ids, list) or not isinstance(raw_cell_levels, list):
        raise MeshImportError("Cell refinement identifiers and levels must be lists.")
    if any(not isinstance(cell_id, str) or not cell_id for cell_id in raw_cell_ids):
        raise MeshImportError("Cell refinement identifiers must be non-empty strings.")
    cell_ids = list(raw_cell_ids)
    cell_levels = [int(v) for v in _integer_array(raw_cell_levels, "Cell refinement levels")]
    if (cell_ids or cell_levels) and not (len(cell_ids) == len(cell_levels) == n_cells):
        raise MeshImportError("Cell refinement metadata has inconsistent lengths.")
    if len(set(cell_ids)) != len(cell_ids) or any(level < 0 for level in cell_levels):
        raise MeshImportError("Cell refinement metadata contains duplicate or negative values.")
    raw_records = raw.get("records", [])
    if not isinstance(raw_records, list):
        raise MeshImportError("Refinement records must be a list.")
    if raw_records and not cell_ids:
        raise MeshImportError("Refinement records require cell identifiers and levels.")
    records, parents = [], set()
    for index, record in enumerate(raw_records):
        if not isinstance(record, dict):
            raise MeshImportError(f"Refinement record {index} must be an object.")
        parent_id = record.get("parent_id")
        child_ids = record.get("child_ids")
        vertices = record.get("vertices")
        level = _integer(record.get("level"), "Refinement parent level")
        if (not isinstance(parent_id, str) or not parent_id or parent_id in parents
                or not isinstance(child_ids, list) or len(child_ids) < 2
                or any(not isinstance(child, str) or not child for child in child_ids)
                or len(set(child_ids)) != len(child_ids)
                or not isinstance(vertices, list) or len(vertices) < 3 or level < 0):
            raise MeshImportError(f"Refinement record {index} is invalid.")
        parents.add(parent_id)
        parsed = []
        for vertex in vertices:
            if not isinstance(vertex, list) or len(vertex) != 2:
                raise MeshImportError(f"Refinement record {index} has invalid vertices.")
            try:
                point = (float(vertex[0]), float(vertex[1]))
            except (OverflowError, TypeError, ValueError) as error:
                raise MeshImportError(f"Refinement record {index} has invalid vertices.") from error
            if not all(math.isfinite(value) for value in point):
                raise MeshImportError(f"Refinement record {index} has non-finite vertices.")
            parsed.append(point)
        records.append(RefinementRecord(parent_id, tuple(child_ids), tuple(parsed), level))
    return tuple(cell_ids), tuple(cell_levels), tuple(records)


# ---------------------------------------------------------------- interface

def mesh_from_dict(data: dict) -> FiniteVolumeMesh:
    """A MeshCAD finite-volume mesh (format ``meshcad-mesh`` version 1) from
    its JSON object; raises MeshImportError with the reference's messages
    (mesh_io.py:133-445)."""
    if data.get("format") != FORMAT_NAME or data.get("version") != FORMAT_VERSION:
        raise MeshImportError(
            f"Unsupported mesh format. Expected MeshCAD finite-volume mesh JSON version {FORMAT_VERSION}.")
    if data.get("dimension") != 2:
        raise MeshImportError("Only two-dimensional meshes are supported.")
    try:
        coordinates = data["nodes"]["coordinates"]
        face_nodes = data["faces"]["nodes"]
        face_owners = data["faces"]["owner"]
        face_neighbours = data["faces"]["neighbour"]
        face_patch_ids = data["faces"]["patch"]
        cell_faces = data["cells"]["faces"]
        cell_signs = data["cells"]["face_signs"]
        raw_patches = data["patches"]
    except (KeyError, TypeError) as error:
        raise MeshImportError(f"Mesh file is missing required data: {error}.") from error

    if not isinstance(coordinates, list) or not coordinates:
        raise MeshImportError("Mesh must contain at least one node.")
    points = _parse_points(coordinates)
    if not isinstance(face_nodes, list) or not face_nodes:
        raise MeshImportError("Mesh must contain at least one face.")
    faces = _parse_faces(face_nodes, len(points))

    owners = _integer_array(face_owners, "Face owners")
    neighbours = _integer_array(face_neighbours, "Face neighbours")
    patch_of_face = _integer_array(face_patch_ids, "Face patch identifiers")
    if not len(faces) == len(owners) == len(neighbours) == len(patch_of_face):
        raise MeshImportError("Face connectivity arrays have inconsistent lengths.")

    patches = _parse_patches(raw_patches, len(faces))
    if not isinstance(cell_faces, list) or not isinstance(cell_signs, list):
        raise MeshImportError("Cell connectivity must be represented by lists.")
    if not cell_faces or len(cell_faces) != len(cell_signs):
        raise MeshImportError("Mesh must have cells with consistent face connectivity.")
    _check_face_links(owners, neighbours, patch_of_face, len(cell_faces), {p.id for p in patches})

    face_curves = ()
    raw_curves = data.get("boundary_curves")
    if raw_curves is not None:
        face_curves = _parse_curves(raw_curves, faces, points, neighbours, patch_of_face)

    cells, cell_face_ids, cell_face_signs = _parse_cells(cell_faces, cell_signs, faces)
    _check_patch_membership(patches, patch_of_face)
    cell_ids, cell_levels, records = _parse_refinement(data.get("refinement", {}), len(cells))

    return FiniteVolumeMesh(
        points=points, cells=cells, faces=faces, face_owners=owners, face_neighbours=neighbours,
        face_patch_ids=patch_of_face, patches=tuple(patches), cell_face_ids=cell_face_ids,
        cell_face_signs=cell_face_signs, cell_ids=cell_ids, cell_levels=cell_levels,
        refinement_records=records, face_curves=face_curves)


def load_mesh(path) -> FiniteVolumeMesh:
    """Read a MeshCAD mesh file (mesh_io.py:448-457)."""
    source = Path(path)
    try:
        with source.open("r", encoding="utf-8") as stream:
            data = json.load(stream)
    except (OSError, UnicodeError, json.JSONDecodeError) as error:
        raise MeshImportError(f"Could not read mesh file '{source}': {error}") from error
    if not isinstance(data, dict):
        raise MeshImportError("Mesh file must contain a JSON object.")
    return mesh_from_dict(data)


def cell_face_lists(mesh: FiniteVolumeMesh):
    """Each cell's faces in its vertex order and their signs (+1 where the
    face's node order follows the cell's), as CSRs (``CellArray``), from the
    cells' vertex loops and the face list: the connectivity the format
    stores, for meshes built without it."""
    from .geometry import _cells_csr

    offsets, nodes = _cells_csr(mesh)
    faces = np.asarray(mesh.faces, dtype=np.int64)
    counts = np.diff(offsets)
    nxt = np.arange(1, len(nodes) + 1, dtype=np.int64)
    nxt[offsets[1:] - 1] = offsets[:-1]  # each cell's last vertex closes the loop
    a, b = nodes, nodes[nxt]
    n = int(max(faces.max(), nodes.max())) + 1
    face_key = np.minimum(faces[:, 0], faces[:, 1]) * n + np.maximum(faces[:, 0], faces[:, 1])
    order = np.argsort(face_key, kind="stable")
    edge_key = np.minimum(a, b) * n + np.maximum(a, b)
    pos = np.minimum(np.searchsorted(face_key[order], edge_key), len(order) - 1)
    if (face_key[order][pos] != edge_key).any():
        raise ValueError("a cell edge has no face")
    face_ids = order[pos]
    signs = np.where(faces[face_ids, 0] == a, 1, -1).astype(np.int64)
    csr = np.concatenate(([0], np.cumsum(counts))).astype(np.int64)
    return CellArray(csr, face_ids.astype(np.int64)), CellArray(csr, signs)


def _rows(csr) -> list:
    offsets = np.asarray(csr.offsets)
    values = np.asarray(csr.nodes).tolist()
    return [values[a:b] for a, b in zip(offsets[:-1].tolist(), offsets[1:].tolist())]


def mesh_to_dict(mesh: FiniteVolumeMesh) -> dict:
    """The mesh as a MeshCAD JSON object, the reference's serialisation
    (mesh_io.py:460-512): same keys, order and value types.  Meshes without
    cell face lists get them from ``cell_face_lists``."""
    cell_face_ids, cell_face_signs = mesh.cell_face_ids, mesh.cell_face_signs
    if len(cell_face_ids) == 0:
        cell_face_ids, cell_face_signs = cell_face_lists(mesh)
    data = {
        "format": FORMAT_NAME,
        "version": FORMAT_VERSION,
        "dimension": 2,
        "nodes": {"coordinates": np.asarray(mesh.points, dtype=np.float64).tolist()},
        "faces": {
            "nodes": np.asarray(mesh.faces).tolist(),
            "owner": np.asarray(mesh.face_owners).tolist(),
            "patch": np.asarray(mesh.face_patch_ids).tolist(),
            "neighbour": np.asarray(mesh.face_neighbours).tolist(),
        },
        "cells": {
            "faces": _rows(cell_face_ids) if hasattr(cell_face_ids, "offsets")
            else [[int(v) for v in ids] for ids in cell_face_ids],
            "face_signs": _rows(cell_face_signs) if hasattr(cell_face_signs, "offsets")
            else [[int(v) for v in signs] for signs in cell_face_signs],
        },
        "patches": [{"id": patch.id, "name": patch.name, "faces": np.asarray(patch.face_ids).tolist()}
                    for patch in mesh.patches],
    }
    if len(mesh.cell_ids) or len(mesh.cell_levels) or len(mesh.refinement_records):
        data["refinement"] = {
            "cell_ids": list(mesh.cell_ids),
            "cell_levels": [int(v) for v in mesh.cell_levels],
            "records": [{"parent_id": r.parent_id, "child_ids": list(r.child_ids),
                         "vertices": [list(point) for point in r.vertices], "level": r.level}
                        for r in mesh.refinement_records],
        }
    if mesh.face_curves:
        if len(mesh.face_curves) != len(mesh.faces):
            raise ValueError("Boundary curve metadata does not match mesh faces.")
        data["boundary_curves"] = [
            None if curve is None else {"geometry": curve.geometry,
                                        "parameters": [curve.start_parameter, curve.end_parameter],
                                        "patch_id": curve.patch_id}
            for curve in mesh.face_curves]
    return data
