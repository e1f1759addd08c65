"""Parity at the full size of the vortex configuration (1024 x 1024 quads,
half split: 1,572,864 cells, HLLC, MUSCL linear, Venkatakrishnan, RK3 at
CFL 0.8): three steps of the device path against the oracle, bit for bit,
where index arithmetic or the time-step minimum over all cells could differ
from the small meshes."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_full_size_vortex_steps_match_the_oracle_bit_for_bit(cuda_device):
    import torch
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, vortex_case, vortex_primitive
    from meshcfd_gb300.solver import run_explicit
    from oracle.oracle import Oracle

    case, _ = vortex_case(1024, split="half")
    g = build_geometry(case.mesh, case)
    assert len(g.areas) == 1572864
    s = case.numerics
    s.flux, s.reconstruction, s.limiter = "HLLC", "MUSCL linear", "Venkatakrishnan"
    s.time_integration, s.cfl = "Explicit RK3", 0.8
    s.end_time, s.max_iterations, s.residual_tolerance = 1.0e30, 3, 1e-300
    orc = Oracle(g)
    U0 = orc.conservative(vortex_primitive(cell_centroids(case.mesh)), s.gamma)
    ref, t_ref = orc.solve(U0, s, 3)
    dg = DeviceGeometry(g)
    U = torch.as_tensor(U0, device=cuda_device)
    result = run_explicit(dg, s, U, final_residual=False)
    assert result.steps == 3 and abs(result.time - t_ref) <= 1e-12 * t_ref
    np.testing.assert_array_equal(U.cpu().numpy(), ref)
