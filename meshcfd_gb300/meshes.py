"""Seeded synthetic meshes and initial states for the benchmark workloads.

The reference ships only a structured unit-square quad generator
(``benchmarks/common.py:53-113``, ``tests/test_solver.py:57-131``).  The meshes
here follow the same face convention: cells are visited in order, each cell's
edges in vertex order, a face is created when an edge is first met (owner =
that cell, orientation = that cell's vertex order) and the second cell to meet
it becomes the neighbour.  Boundary faces are assigned to patches by position.
All builders are vectorised so that multi-million-cell meshes take seconds.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .model import (
    BoundaryCondition,
    Case,
    FiniteVolumeMesh,
    InitialState,
    MeshPatch,
    PeriodicBoundaryPair,
)


@dataclass
class CellArray:
    """Cells as a vertex CSR: cell ``c`` has vertices ``nodes[offsets[c]:offsets[c+1]]``."""

    offsets: np.ndarray
    nodes: np.ndarray

    def __len__(self) -> int:
        return len(self.offsets) - 1

    def __iter__(self):
        for c in range(len(self)):
            yield tuple(int(v) for v in self.nodes[self.offsets[c]:self.offsets[c + 1]])

    def __getitem__(self, c):
        return tuple(int(v) for v in self.nodes[self.offsets[c]:self.offsets[c + 1]])


def build_faces(points: np.ndarray, cells: CellArray, classify) -> FiniteVolumeMesh:
    """Create faces, owners, neighbours and patches from cell vertex lists.

    ``classify(a, b)`` maps the boundary edge end points (arrays (n,2)) to patch
    ids (>= 0), returning a tuple ``(patch_ids, patch_names)``.
    """
    offsets = np.asarray(cells.offsets, dtype=np.int64)
    nodes = np.asarray(cells.nodes, dtype=np.int64)
    counts = np.diff(offsets)
    n_cells = len(counts)
    edge_cell = np.repeat(np.arange(n_cells, dtype=np.int64), counts)
    position = np.arange(len(nodes), dtype=np.int64)
    last = offsets[1:] - 1
    next_index = position + 1
    next_index[last] = offsets[:-1]
    start = nodes
    end = nodes[next_index]
    n_points = len(points)
    key = np.minimum(start, end) * n_points + np.maximum(start, end)
    _, first, inverse = np.unique(key, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    face_of_edge = rank[inverse]
    first_sorted = first[order]
    faces = np.column_stack((start[first_sorted], end[first_sorted]))
    owners = edge_cell[first_sorted]
    neighbours = np.full(len(faces), -1, dtype=np.int64)
    is_first = np.zeros(len(nodes), dtype=bool)
    is_first[first_sorted] = True
    second = ~is_first
    if np.any(np.bincount(face_of_edge, minlength=len(faces)) > 2):
        raise ValueError("non-manifold edge: more than two cells share a face")
    neighbours[face_of_edge[second]] = edge_cell[second]
    boundary = np.flatnonzero(neighbours < 0)
    patch_ids = np.full(len(faces), -1, dtype=np.int64)
    ids, names = classify(points[faces[boundary, 0]], points[faces[boundary, 1]])
    patch_ids[boundary] = ids
    if np.any(patch_ids[boundary] < 0):
        raise ValueError("boundary face without a patch")
    patches = tuple(
        MeshPatch(pid, name, tuple(int(f) for f in boundary[ids == pid]))
        for pid, name in enumerate(names)
    )
    signs = np.where(owners[face_of_edge] == edge_cell, 1, -1)
    return FiniteVolumeMesh(
        points=np.asarray(points, dtype=np.float64),
        cells=cells,
        faces=faces,
        face_owners=owners,
        face_neighbours=neighbours,
        face_patch_ids=patch_ids,
        patches=patches,
        cell_face_ids=CellArray(offsets, face_of_edge),
        cell_face_signs=CellArray(offsets, signs),
    )


def permute_mesh(mesh: FiniteVolumeMesh, cell_order=None, face_order=None) -> FiniteVolumeMesh:
    """The same mesh with other cell and face ids: new cell k is old cell
    ``cell_order[k]``, new face k is old face ``face_order[k]`` (None keeps
    the ids).  Owners, neighbours, face orientation and the patches' face
    order are carried over, so the geometry is the same up to the ids (a
    mesh read from a file arrives in whatever order the file has)."""
    offsets = np.asarray(mesh.cells.offsets, dtype=np.int64)
    nodes = np.asarray(mesh.cells.nodes, dtype=np.int64)
    n_cells, n_faces = len(offsets) - 1, len(mesh.faces)
    co = np.arange(n_cells) if cell_order is None else np.asarray(cell_order, dtype=np.int64)
    fo = np.arange(n_faces) if face_order is None else np.asarray(face_order, dtype=np.int64)
    inv_c = np.empty(n_cells, dtype=np.int64)
    inv_c[co] = np.arange(n_cells)
    inv_f = np.empty(n_faces, dtype=np.int64)
    inv_f[fo] = np.arange(n_faces)
    counts = np.diff(offsets)[co]
    new_offsets = np.concatenate(([0], np.cumsum(counts))).astype(np.int64)
    take = np.concatenate([np.arange(offsets[c], offsets[c + 1]) for c in co]) if n_cells else np.empty(0, np.int64)
    owners = inv_c[np.asarray(mesh.face_owners, dtype=np.int64)[fo]]
    nb = np.asarray(mesh.face_neighbours, dtype=np.int64)[fo]
    neighbours = np.where(nb >= 0, inv_c[np.maximum(nb, 0)], -1)
    face_ids = np.asarray(mesh.cell_face_ids.nodes, dtype=np.int64)[take]
    signs = np.asarray(mesh.cell_face_signs.nodes)[take]
    return FiniteVolumeMesh(
        points=mesh.points,
        cells=CellArray(new_offsets, nodes[take]),
        faces=np.asarray(mesh.faces)[fo],
        face_owners=owners,
        face_neighbours=neighbours,
        face_patch_ids=np.asarray(mesh.face_patch_ids)[fo],
        patches=tuple(MeshPatch(p.id, p.name, tuple(int(inv_f[f]) for f in p.face_ids)) for p in mesh.patches),
        cell_face_ids=CellArray(new_offsets, inv_f[face_ids]),
        cell_face_signs=CellArray(new_offsets, signs),
    )


def reverse_cuthill_mckee(mesh: FiniteVolumeMesh) -> tuple[np.ndarray, np.ndarray]:
    """Cell and face orders that number the mesh by reverse Cuthill-McKee
    (breadth-first from a minimum-degree cell, neighbours by increasing
    degree, reversed), faces then by their smaller new cell id.  For
    :func:`permute_mesh`."""
    owners = np.asarray(mesh.face_owners, dtype=np.int64)
    nbs = np.asarray(mesh.face_neighbours, dtype=np.int64)
    n = len(mesh.cells.offsets) - 1
    inner = nbs >= 0
    a = np.concatenate((owners[inner], nbs[inner]))
    b = np.concatenate((nbs[inner], owners[inner]))
    order = np.lexsort((b, a))
    a, b = a[order], b[order]
    ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(ptr, a + 1, 1)
    ptr = np.cumsum(ptr)
    degree = np.diff(ptr)
    seen = np.zeros(n, dtype=bool)
    out = np.empty(n, dtype=np.int64)
    k = 0
    for start in np.argsort(degree, kind="stable"):
        if seen[start]:
            continue
        seen[start] = True
        out[k] = start
        head, k = k, k + 1
        while head < k:
            c = out[head]
            head += 1
            nb = b[ptr[c]:ptr[c + 1]]
            nb = nb[~seen[nb]]
            if len(nb):
                nb = np.unique(nb)
                nb = nb[np.argsort(degree[nb], kind="stable")]
                seen[nb] = True
                out[k:k + len(nb)] = nb
                k += len(nb)
    cell_order = out[::-1].copy()
    new_id = np.empty(n, dtype=np.int64)
    new_id[cell_order] = np.arange(n)
    key = np.where(inner, np.minimum(new_id[owners], new_id[np.maximum(nbs, 0)]), new_id[owners])
    face_order = np.lexsort((np.where(inner, np.maximum(new_id[owners], new_id[np.maximum(nbs, 0)]), -1), key))
    return cell_order, face_order


def renumber_cells(mesh: FiniteVolumeMesh) -> tuple[FiniteVolumeMesh, np.ndarray]:
    """The mesh with its cells renumbered by reverse Cuthill-McKee and its
    faces left in their order; returns (mesh, cell_order), new cell k being
    old cell ``cell_order[k]``.

    Every per-cell sum of the explicit path runs over the cell's entries in
    face order (gradient entries, limiter entries, divergence, boundary
    groups, time-step entries), so with the faces kept the renumbered mesh
    gives the same values bit for bit, cell by cell: ``R_new ==
    R_old[cell_order]``.  Neighbouring cells then sit close in memory,
    which is what the per-cell kernels gather by (a mesh file may number its
    cells in any order).  Not for the implicit path: its LU-SGS sweeps follow
    the cell numbering (solver.py:1302-1323), so renumbering changes the
    preconditioner."""
    cell_order, _ = reverse_cuthill_mckee(mesh)
    return permute_mesh(mesh, cell_order, None), cell_order


def to_reference_mesh(mesh: FiniteVolumeMesh, mesh_type):
    """Convert to the reference's tuple-based ``FiniteVolumeMesh`` (small meshes)."""
    patch_type = type(mesh.patches[0]) if mesh.patches else None
    return mesh_type(
        points=tuple((float(x), float(y)) for x, y in np.asarray(mesh.points)),
        cells=tuple(tuple(c) for c in mesh.cells),
        faces=tuple((int(a), int(b)) for a, b in np.asarray(mesh.faces)),
        face_owners=tuple(int(v) for v in mesh.face_owners),
        face_neighbours=tuple(int(v) for v in mesh.face_neighbours),
        face_patch_ids=tuple(int(v) for v in mesh.face_patch_ids),
        patches=tuple(p for p in mesh.patches) if patch_type is None else mesh.patches,
        cell_face_ids=tuple(tuple(c) for c in mesh.cell_face_ids),
        cell_face_signs=tuple(tuple(c) for c in mesh.cell_face_signs),
    )


def _grid_points(nx, ny, x0, x1, y0, y1):
    xs = x0 + (x1 - x0) * np.arange(nx + 1) / nx
    ys = y0 + (y1 - y0) * np.arange(ny + 1) / ny
    gx, gy = np.meshgrid(xs, ys)
    points = np.column_stack((gx.ravel(), gy.ravel()))
    # exact boundary coordinates, so that periodic patches match bit for bit
    points[np.isclose(points[:, 0], x1), 0] = x1
    points[np.isclose(points[:, 1], y1), 1] = y1
    return points


def _jitter_interior(points, nx, ny, hx, hy, amplitude, rng):
    j, i = np.divmod(np.arange(len(points)), nx + 1)
    interior = (i > 0) & (i < nx) & (j > 0) & (j < ny)
    shift = rng.uniform(-amplitude, amplitude, size=(int(interior.sum()), 2))
    points = points.copy()
    points[interior, 0] += shift[:, 0] * hx
    points[interior, 1] += shift[:, 1] * hy
    return points


def _split_cells(nx, ny, split_mask):
    """Quads in row-major order; a split quad becomes two consecutive triangles
    sharing its bottom-left to top-right diagonal (both counter-clockwise)."""
    j, i = np.divmod(np.arange(nx * ny), nx)
    bl = j * (nx + 1) + i
    br = bl + 1
    tr = br + nx + 1
    tl = bl + nx + 1
    counts = np.where(split_mask, 6, 4)
    nodes = np.empty(int(counts.sum()), dtype=np.int64)
    starts = np.concatenate(([0], np.cumsum(counts)[:-1]))
    quad = ~split_mask
    for k, v in enumerate((bl, br, tr, tl)):
        nodes[starts[quad] + k] = v[quad]
    for k, v in enumerate((bl, br, tr, bl, tr, tl)):
        nodes[starts[split_mask] + k] = v[split_mask]
    cell_counts = np.repeat(np.where(split_mask, 3, 4), np.where(split_mask, 2, 1))
    offsets = np.concatenate(([0], np.cumsum(cell_counts))).astype(np.int64)
    return CellArray(offsets, nodes)


def _box_classifier(x0, x1, y0, y1):
    names = ("bottom", "right", "top", "left")

    def classify(a, b):
        ids = np.full(len(a), -1, dtype=np.int64)
        ids[(a[:, 1] == y0) & (b[:, 1] == y0)] = 0
        ids[(a[:, 0] == x1) & (b[:, 0] == x1)] = 1
        ids[(a[:, 1] == y1) & (b[:, 1] == y1)] = 2
        ids[(a[:, 0] == x0) & (b[:, 0] == x0)] = 3
        return ids, names

    return classify


def box_mesh(nx, ny, lx=1.0, ly=1.0, split="none", jitter=0.0, seed=0, x0=0.0, y0=0.0, separate_left=False):
    """Rectangle [x0,x0+lx]x[y0,y0+ly] of nx*ny quads.

    ``split``: "none" (quads), "all" (two triangles per quad) or "half" (a
    seed-chosen half of the quads, exactly nx*ny//2 of them, are split).
    ``jitter``: interior vertices move uniformly by up to +-jitter*h per axis.
    ``separate_left``: every face of the left side is a patch of its own
    ("left0" bottom to "left{ny-1}" top) instead of one "left" patch.
    """
    x1, y1 = x0 + lx, y0 + ly
    rng = np.random.default_rng(seed)
    points = _grid_points(nx, ny, x0, x1, y0, y1)
    if split == "none":
        mask = np.zeros(nx * ny, dtype=bool)
    elif split == "all":
        mask = np.ones(nx * ny, dtype=bool)
    elif split == "half":
        mask = np.zeros(nx * ny, dtype=bool)
        mask[rng.permutation(nx * ny)[: (nx * ny) // 2]] = True
    else:
        raise ValueError(split)
    if jitter:
        points = _jitter_interior(points, nx, ny, lx / nx, ly / ny, jitter, rng)
    cells = _split_cells(nx, ny, mask)
    classify = _box_classifier(x0, x1, y0, y1)
    if separate_left:
        base = classify

        def classify(a, b):
            ids, names = base(a, b)
            left = np.flatnonzero(ids == 3)
            rank = np.argsort(np.argsort(a[left, 1] + b[left, 1], kind="stable"), kind="stable")
            ids = ids.copy()
            ids[left] = 3 + rank
            return ids, names[:3] + tuple(f"left{k}" for k in range(len(left)))

    return build_faces(points, cells, classify)


# ---------------------------------------------------------------- workloads

RIEMANN_QUADRANTS = (
    # (rho, u, v, p) for x>0.5,y>0.5 / x<0.5,y>0.5 / x<0.5,y<0.5 / x>0.5,y<0.5
    (1.5, 0.0, 0.0, 1.5),
    (0.5323, 1.206, 0.0, 0.3),
    (0.138, 1.206, 1.206, 0.029),
    (0.5323, 0.0, 1.206, 0.3),
)


def cell_centroids(mesh) -> np.ndarray:
    """Vertex averages (used only to place initial conditions)."""
    cells = mesh.cells
    pts = np.asarray(mesh.points)
    offsets, nodes = cells.offsets, cells.nodes
    counts = np.diff(offsets)
    owner = np.repeat(np.arange(len(counts)), counts)
    cx = np.bincount(owner, weights=pts[nodes, 0]) / counts
    cy = np.bincount(owner, weights=pts[nodes, 1]) / counts
    return np.column_stack((cx, cy))


def riemann_case(n=128, seed=0, jitter=0.2):
    """Four-quadrant 2D Riemann problem on a jittered triangulated unit square.

    Walls top and bottom, far field left and right.  The far-field state on each
    side is the initial state of the quadrant pair it touches, averaged over the
    two quadrants of that side (left: quadrants 1,2; right: 0,3)."""
    mesh = box_mesh(n, n, 1.0, 1.0, split="all", jitter=jitter, seed=seed)
    case = Case(name=f"riemann{n}", mesh=mesh)
    s = RIEMANN_QUADRANTS
    left = tuple(0.5 * (a + b) for a, b in zip(s[1], s[2]))
    right = tuple(0.5 * (a + b) for a, b in zip(s[0], s[3]))
    for condition in case.boundary_conditions:
        if condition.patch_name in ("bottom", "top"):
            condition.kind = "Wall"
            condition.mechanical_condition = "Slip"
        else:
            st = left if condition.patch_name == "left" else right
            condition.kind = "Far Field"
            condition.values = {"density": st[0], "velocity_x": st[1], "velocity_y": st[2], "pressure": st[3]}
    num = case.numerics
    num.flux, num.reconstruction = "Rusanov", "First order"
    num.time_integration, num.cfl = "Explicit Euler", 0.5
    num.end_time, num.max_iterations = 1.0e30, 100
    num.residual_tolerance = 1e-300
    centers = cell_centroids(mesh)
    east = centers[:, 0] > 0.5
    north = centers[:, 1] > 0.5
    quadrant = np.where(north, np.where(east, 0, 1), np.where(east, 3, 2))
    primitive = np.asarray(s, dtype=np.float64)[quadrant]
    return case, primitive


def vortex_primitive(centers, t=0.0, beta=5.0, mach=0.5, angle_deg=45.0, gamma=1.4,
                     center=(5.0, 5.0), period=(10.0, 10.0)):
    """Isentropic vortex (strength beta) advected by a free stream of Mach
    ``mach`` at ``angle_deg``; exact solution at time ``t`` on the periodic box."""
    speed = mach * math.sqrt(gamma)  # free stream rho=1, p=1, so c = sqrt(gamma)
    ux = speed * math.cos(math.radians(angle_deg))
    uy = speed * math.sin(math.radians(angle_deg))
    cx = (center[0] + ux * t) % period[0]
    cy = (center[1] + uy * t) % period[1]
    dx = centers[:, 0] - cx
    dy = centers[:, 1] - cy
    dx -= period[0] * np.round(dx / period[0])
    dy -= period[1] * np.round(dy / period[1])
    r2 = dx * dx + dy * dy
    ex = np.exp(0.5 * (1.0 - r2))
    temperature = 1.0 - (gamma - 1.0) * beta**2 / (8.0 * gamma * math.pi**2) * np.exp(1.0 - r2)
    rho = temperature ** (1.0 / (gamma - 1.0))
    u = ux - beta / (2.0 * math.pi) * ex * dy
    v = uy + beta / (2.0 * math.pi) * ex * dx
    p = rho**gamma
    return np.column_stack((rho, u, v, p))


def vortex_case(n=1024, seed=0, jitter=0.15, split="half", length=10.0):
    """Isentropic vortex on a periodic [0,L]^2 box of n*n quads, a seed-chosen
    half of them split into triangles (split="all": every quad split)."""
    mesh = box_mesh(n, n, length, length, split=split, jitter=jitter, seed=seed)
    case = Case(name=f"vortex{n}", mesh=mesh)
    for condition in case.boundary_conditions:
        condition.kind = "Periodic"
    case.periodic_pairs = [
        PeriodicBoundaryPair(1, 3, "x", length),
        PeriodicBoundaryPair(0, 2, "y", length),
    ]
    num = case.numerics
    num.flux, num.reconstruction, num.limiter = "HLLC", "MUSCL linear", "Venkatakrishnan"
    num.time_integration, num.cfl = "Explicit RK3", 0.8
    num.end_time, num.max_iterations = 1.0e30, 100
    num.residual_tolerance = 1e-300
    return case, None


def periodic_case(nx, ny, lx=1.0, ly=1.0, split="none", jitter=0.0, seed=0):
    mesh = box_mesh(nx, ny, lx, ly, split=split, jitter=jitter, seed=seed)
    case = Case(name="periodic", mesh=mesh)
    for condition in case.boundary_conditions:
        condition.kind = "Periodic"
    case.periodic_pairs = [
        PeriodicBoundaryPair(1, 3, "x", lx),
        PeriodicBoundaryPair(0, 2, "y", ly),
    ]
    return case


def smooth_primitive(n_cells, seed=0, amplitude=0.05):
    """A smooth, positive, non-uniform state keyed by cell id (as the reference
    benchmark does, benchmarks/common.py:128-140) plus a seeded perturbation."""
    cell = np.arange(n_cells, dtype=np.float64)
    rng = np.random.default_rng(seed)
    noise = rng.uniform(-1.0, 1.0, size=(n_cells, 4)) * amplitude * 0.1
    rho = 1.0 + 0.02 * np.sin(0.017 * cell) + noise[:, 0]
    u = 0.20 + 0.03 * np.sin(0.011 * cell) + noise[:, 1]
    v = 0.03 * np.cos(0.013 * cell) + noise[:, 2]
    p = 1.0 + 0.02 * np.cos(0.019 * cell) + noise[:, 3]
    return np.column_stack((rho, u, v, p))


def states_from_primitive(primitive) -> tuple:
    return tuple(InitialState(*map(float, row)) for row in np.asarray(primitive))


def ogrid_case(n_theta=1024, n_r=512, radius=0.5, half_width=10.0, growth=None, seed=2, jitter=0.1, mach=0.3):
    """O-grid of n_theta x n_r quads around a cylinder of ``radius`` centred in
    the square [-half_width, half_width]^2: radial lines from the circle to the
    square, points spaced geometrically along them (ratio ``growth``, default
    chosen so the first spacing is ~ the circumferential spacing at the wall),
    interior points jittered by up to ``jitter`` of the local spacing (seeded).
    Slip wall on the cylinder, far field (free stream at Mach ``mach`` along x,
    rho = 1, p = 1/gamma... p = 1) on the square."""
    rng = np.random.default_rng(seed)
    theta = 2.0 * math.pi * np.arange(n_theta) / n_theta
    c, s = np.cos(theta), np.sin(theta)
    inner = radius * np.column_stack((c, s))
    scale = half_width / np.maximum(np.abs(c), np.abs(s))
    outer = scale[:, None] * np.column_stack((c, s))
    if growth is None:
        first = 2.0 * math.pi * radius / n_theta
        span = float(np.min(scale)) - radius
        lo, hi = 1.0 + 1e-9, 2.0
        for _ in range(100):  # first spacing span*(g-1)/(g^n-1) = first
            g = 0.5 * (lo + hi)
            if span * (g - 1.0) / (g**n_r - 1.0) > first:
                lo = g
            else:
                hi = g
        growth = 0.5 * (lo + hi)
    t = (growth ** np.arange(n_r + 1) - 1.0) / (growth**n_r - 1.0)
    pts = inner[None, :, :] + t[:, None, None] * (outer - inner)[None, :, :]
    if jitter:
        dt = np.diff(t)
        h_r = np.minimum(dt[:-1], dt[1:])[:, None] * np.linalg.norm(outer - inner, axis=1)[None, :]
        h_t = 2.0 * math.pi * np.linalg.norm(pts[1:-1], axis=2) / n_theta
        h = np.minimum(h_r, h_t)
        pts[1:-1] += (rng.uniform(-jitter, jitter, size=(n_r - 1, n_theta, 2)) * h[:, :, None])
    points = pts.reshape(-1, 2)
    j, i = np.divmod(np.arange(n_theta * n_r), n_theta)
    ip = (i + 1) % n_theta
    quad = np.column_stack((j * n_theta + i, j * n_theta + ip, (j + 1) * n_theta + ip, (j + 1) * n_theta + i))
    cells = CellArray(np.arange(0, 4 * len(quad) + 1, 4, dtype=np.int64), quad.ravel().astype(np.int64))
    def classify(a, b):
        ra = np.linalg.norm(a, axis=1)
        ids = np.where(ra < 0.5 * (radius + half_width), 0, 1)
        return ids, ("cylinder", "farfield")

    mesh = build_faces(points, cells, classify)
    case = Case(name=f"ogrid{n_theta}x{n_r}", mesh=mesh)
    gamma = case.numerics.gamma
    u = mach * math.sqrt(gamma)
    for cond in case.boundary_conditions:
        if cond.patch_name == "cylinder":
            cond.kind = "Wall"
            cond.mechanical_condition = "Slip"
        else:
            cond.kind = "Far Field"
            cond.values = {"density": 1.0, "velocity_x": u, "velocity_y": 0.0, "pressure": 1.0}
    num = case.numerics
    num.flux, num.reconstruction, num.limiter = "HLLC", "MUSCL linear", "Venkatakrishnan"
    num.time_integration, num.cfl = "Explicit RK3", 0.8
    num.time_step_mode, num.end_time, num.residual_tolerance = "Global fixed", 1.0e30, 1e-300
    P = np.tile((1.0, u, 0.0, 1.0), (len(mesh.cells), 1))
    return case, P


def bump_case(nx=512, ny=256, height=0.1, seed=1, stretch=1.05, jitter=0.1, mach=0.5, x0=-1.0, x1=2.0, top=1.0):
    """Channel over a circular-arc bump: x in [x0, x1] with the arc of chord 1
    (x from 0 to 1) and ``height`` on the lower wall, the upper boundary at
    y = ``top``; nx x ny quads, rows spaced geometrically from the lower wall
    (ratio ``stretch``), interior points jittered by up to ``jitter`` of the
    local spacing (seeded).  Slip wall below, far field (free stream at Mach
    ``mach`` along x, rho = 1, p = 1) at the inflow and on top, pressure
    outlet (p = 1) at the outflow.  Settings: Roe, MUSCL linear with
    Barth-Jespersen, implicit Euler with local time steps at CFL 200,
    GMRES(30) to 1e-3 with LU-SGS."""
    rng = np.random.default_rng(seed)
    xs = x0 + (x1 - x0) * np.arange(nx + 1) / nx
    xs[-1] = x1
    radius = (0.25 + height * height) / (2.0 * height)
    on_arc = (xs > 0.0) & (xs < 1.0)
    yb = np.zeros(nx + 1)
    yb[on_arc] = np.sqrt(radius * radius - (xs[on_arc] - 0.5) ** 2) - (radius - height)
    t = (stretch ** np.arange(ny + 1) - 1.0) / (stretch**ny - 1.0)
    t[-1] = 1.0
    X = np.broadcast_to(xs, (ny + 1, nx + 1)).copy()
    Y = yb[None, :] + t[:, None] * (top - yb)[None, :]
    Y[-1, :] = top
    if jitter:
        dy = np.diff(Y, axis=0)
        h = np.minimum(np.minimum(dy[:-1], dy[1:]), (x1 - x0) / nx)[:, 1:-1]
        shift = rng.uniform(-jitter, jitter, size=(ny - 1, nx - 1, 2)) * h[:, :, None]
        X[1:-1, 1:-1] += shift[:, :, 0]
        Y[1:-1, 1:-1] += shift[:, :, 1]
    points = np.column_stack((X.ravel(), Y.ravel()))
    j, i = np.divmod(np.arange(nx * ny), nx)
    bl = j * (nx + 1) + i
    quad = np.column_stack((bl, bl + 1, bl + nx + 2, bl + nx + 1))
    cells = CellArray(np.arange(0, 4 * len(quad) + 1, 4, dtype=np.int64), quad.ravel().astype(np.int64))

    def classify(a, b):
        ids = np.zeros(len(a), dtype=np.int64)  # the lower wall
        ids[(a[:, 0] == x0) & (b[:, 0] == x0)] = 1
        ids[(a[:, 1] == top) & (b[:, 1] == top)] = 2
        ids[(a[:, 0] == x1) & (b[:, 0] == x1)] = 3
        return ids, ("wall", "inflow", "top", "outflow")

    mesh = build_faces(points, cells, classify)
    case = Case(name=f"bump{nx}x{ny}", mesh=mesh)
    u = mach * math.sqrt(case.numerics.gamma)
    for cond in case.boundary_conditions:
        if cond.patch_name == "wall":
            cond.kind = "Wall"
            cond.mechanical_condition = "Slip"
        elif cond.patch_name == "outflow":
            cond.kind = "Pressure Outlet"
            cond.values = {"pressure": 1.0}
        else:
            cond.kind = "Far Field"
            cond.values = {"density": 1.0, "velocity_x": u, "velocity_y": 0.0, "pressure": 1.0}
    num = case.numerics
    num.flux, num.reconstruction, num.limiter = "Roe", "MUSCL linear", "Barth-Jespersen"
    num.time_integration, num.cfl, num.time_step_mode = "Implicit Euler", 200.0, "Local (steady)"
    num.gmres_tolerance, num.gmres_krylov_dimension, num.implicit_preconditioner = 1e-3, 30, "LU-SGS"
    num.end_time, num.residual_tolerance = 1.0e30, 1e-300
    P = np.tile((1.0, u, 0.0, 1.0), (len(mesh.cells), 1))
    return case, P

