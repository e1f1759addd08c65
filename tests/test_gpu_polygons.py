"""Cells with more than four faces (pentagons and hexagons from nodes
inserted on interior edges of a periodic quad / triangle mesh): the fast
reconstruction handles them in its separate any-count kernel, and the
residual matches the oracle -- bit for bit for the min limiters, within the
residual bar for the others."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_RESIDUAL = 1e-12


def _polygon_case(nx=10, ny=8, seed=3):
    """Periodic [0,1]^2 mesh: half the quads split into triangles; on three
    vertical edges between unsplit quads one node is inserted (two
    pentagons each), on one edge two nodes (two hexagons)."""
    from meshcfd_gb300.meshes import CellArray, _box_classifier, _grid_points, _split_cells, build_faces
    from meshcfd_gb300.model import Case, PeriodicBoundaryPair

    rng = np.random.default_rng(seed)
    mask = np.zeros(nx * ny, dtype=bool)
    mask[rng.permutation(nx * ny)[: nx * ny // 2]] = True
    pairs = []
    for j in range(1, ny - 1):
        for i in range(1, nx - 2):
            a, b = j * nx + i, j * nx + i + 1
            if not mask[a] and not mask[b] and all(abs(a - p) > 2 and abs(b - q) > 2 for p, q in pairs):
                pairs.append((a, b))
    pairs = pairs[:4]
    assert len(pairs) == 4
    base = _split_cells(nx, ny, mask)
    cells = [list(c) for c in base]
    # quads only (unsplit) map to one cell each: cell index of quad q
    quad_cell = np.cumsum(np.where(mask, 2, 1)) - np.where(mask, 2, 1)
    points = _grid_points(nx, ny, 0.0, 1.0, 0.0, 1.0)
    h = 1.0 / nx
    extra = []
    for k, (qa, qb) in enumerate(pairs):
        left, right = cells[quad_cell[qa]], cells[quad_cell[qb]]  # (bl, br, tr, tl)
        br, tr = left[1], left[2]
        n_new = 2 if k == 0 else 1
        new_ids = []
        for m in range(n_new):
            t = (m + 1) / (n_new + 1)
            p = (1 - t) * points[br] + t * points[tr] + np.array([0.1 * h * (1 if m else -1), 0.0])
            new_ids.append(len(points) + len(extra))
            extra.append(p)
        cells[quad_cell[qa]] = [left[0], left[1], *new_ids, left[2], left[3]]
        cells[quad_cell[qb]] = [right[0], right[1], right[2], right[3], *reversed(new_ids)]
    points = np.vstack([points, np.array(extra)])
    counts = np.array([len(c) for c in cells])
    offsets = np.concatenate(([0], np.cumsum(counts))).astype(np.int64)
    mesh = build_faces(points, CellArray(offsets, np.concatenate([np.array(c) for c in cells]).astype(np.int64)),
                       _box_classifier(0.0, 1.0, 0.0, 1.0))
    case = Case(name="polygons", mesh=mesh)
    for condition in case.boundary_conditions:
        condition.kind = "Periodic"
    case.periodic_pairs = [PeriodicBoundaryPair(1, 3, "x", 1.0), PeriodicBoundaryPair(0, 2, "y", 1.0)]
    return case


@pytest.mark.parametrize("flux", ("Rusanov", "HLLC", "Roe"))
@pytest.mark.parametrize("limiter", ("Barth-Jespersen", "Minmod", "Van Leer", "Venkatakrishnan"))
def test_polygon_cells_match_the_oracle(cuda_device, flux, limiter):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, vortex_primitive
    from meshcfd_gb300.model import NumericalSettings
    from oracle.oracle import Oracle

    case = _polygon_case()
    g = build_geometry(case.mesh, case)
    counts = np.bincount(np.asarray(g.limiter_cells), minlength=len(g.areas))
    assert (counts == 5).sum() == 6 and (counts == 6).sum() == 2
    orc = Oracle(g)
    P = vortex_primitive(10.0 * cell_centroids(case.mesh), mach=0.3)  # the vortex's [0, 10]^2 frame
    P[:, 0] *= 1.0 + 0.05 * np.sin(7.0 * np.arange(len(P)))
    U = orc.conservative(P, 1.4)
    dg = DeviceGeometry(g)
    s = NumericalSettings(flux=flux, reconstruction="MUSCL linear", limiter=limiter)
    ref = orc.residual(U, s)
    for mode in ("fast", "exact"):
        R = dg.residual(torch.as_tensor(U, device=cuda_device), make_config(s, mode=mode)).cpu().numpy()
        dg.check_status()
        if mode == "exact" or limiter in ("Barth-Jespersen", "Minmod"):
            np.testing.assert_array_equal(R, ref)
        else:
            assert np.abs(R - ref).max() <= TOL_RESIDUAL * np.abs(ref).max()
