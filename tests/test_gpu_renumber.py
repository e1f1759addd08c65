"""Cell renumbering on the device: an arbitrarily (randomly) numbered mesh
and the same mesh with its cells renumbered by reverse Cuthill-McKee
(meshes.renumber_cells, faces kept) give each cell's residual and state
after RK3 steps bit for bit, in every kernel variant."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("mode", ("exact", "fast", "fma"))
def test_renumbered_cells_give_the_same_bits_on_the_device(cuda_device, mode):
    from copy import deepcopy

    from meshcfd_gb300.device import DeviceGeometry, make_config, primitive_to_conservative
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, permute_mesh, renumber_cells, vortex_case, vortex_primitive
    from meshcfd_gb300.solver import run_explicit

    case, _ = vortex_case(64, split="half")
    rng = np.random.default_rng(3)
    case.mesh = permute_mesh(case.mesh, rng.permutation(len(case.mesh.cells)), rng.permutation(len(case.mesh.faces)))
    P = vortex_primitive(cell_centroids(case.mesh))
    case2 = deepcopy(case)
    case2.mesh, order = renumber_cells(case.mesh)
    s = case.numerics
    s.max_iterations = 5
    out = []
    for c, Pc in ((case, P), (case2, P[order])):
        dg = DeviceGeometry(build_geometry(c.mesh, c))
        U = torch.as_tensor(primitive_to_conservative(Pc, s.gamma), device=cuda_device)
        R = dg.residual(U, make_config(s, mode)).cpu().numpy()
        res = run_explicit(dg, s, U, mode=mode, final_residual=False)
        out.append((R, U.cpu().numpy(), res.time))
        dg.close()
    np.testing.assert_array_equal(out[1][0], out[0][0][order])
    np.testing.assert_array_equal(out[1][1], out[0][1][order])
    assert out[1][2] == out[0][2]
