"""Cell renumbering (meshes.renumber_cells): reverse Cuthill-McKee on the
cells of an arbitrarily numbered mesh, faces left in their order.  Every
per-cell sum of the explicit path runs over the cell's entries in face
order, so the renumbered mesh gives each cell's residual, time step and
state after RK3 steps bit for bit (checked on the oracle, which follows the
reference's loops; the device's equality is in test_gpu_renumber.py)."""

import numpy as np
import pytest


def _meshes(n=24, seed=7):
    from meshcfd_gb300.meshes import cell_centroids, permute_mesh, renumber_cells, vortex_case, vortex_primitive

    case, _ = vortex_case(n, split="half")
    rng = np.random.default_rng(seed)
    case.mesh = permute_mesh(case.mesh, rng.permutation(len(case.mesh.cells)), rng.permutation(len(case.mesh.faces)))
    P = vortex_primitive(cell_centroids(case.mesh))
    mesh2, order = renumber_cells(case.mesh)
    return case, P, mesh2, order


def test_renumbered_cells_are_a_bandwidth_reducing_permutation():
    case, _, mesh2, order = _meshes()
    assert sorted(order) == list(range(len(order)))

    def bandwidth(m):
        o, nb = np.asarray(m.face_owners), np.asarray(m.face_neighbours)
        inner = nb >= 0
        return int(np.max(np.abs(o[inner] - nb[inner])))

    assert bandwidth(mesh2) < bandwidth(case.mesh) // 10
    np.testing.assert_array_equal(np.asarray(mesh2.faces), np.asarray(case.mesh.faces))


@pytest.mark.parametrize("limiter", ("Venkatakrishnan", "Barth-Jespersen"))
def test_renumbered_cells_give_the_same_bits_on_the_oracle(limiter):
    from copy import deepcopy

    from meshcfd_gb300.geometry import build_geometry
    from oracle.oracle import Oracle

    case, P, mesh2, order = _meshes()
    case.numerics.limiter = limiter
    case2 = deepcopy(case)
    case2.mesh = mesh2
    o1, o2 = Oracle(build_geometry(case.mesh, case)), Oracle(build_geometry(mesh2, case2))
    s = case.numerics
    U1, U2 = o1.conservative(P, s.gamma), o2.conservative(P[order], s.gamma)
    np.testing.assert_array_equal(o2.residual(U2, s), o1.residual(U1, s)[order])
    np.testing.assert_array_equal(o2.stable_time_steps(P[order], s), o1.stable_time_steps(P, s)[order])
    V1, t1 = o1.solve(U1, s, 5)
    V2, t2 = o2.solve(U2, s, 5)
    assert t1 == t2
    np.testing.assert_array_equal(V2, V1[order])
