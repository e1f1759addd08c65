"""Explicit stages as one cooperative launch (mcfd_set_fused_stage): the
reconstruction, face-flux and gather phases of a stage in one resident grid
with grid barriers between them give the same bits as one launch per kernel,
for every time scheme the fused kernel takes (Euler, SSP-RK2, SSP-RK3) and
falls back to the launch per kernel elsewhere (SSPRK(5,4), the exact
variant), on periodic meshes and on a batch with walls and far field."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _vortex(split, limiter, cuda_device):
    from meshcfd_gb300.device import DeviceGeometry, primitive_to_conservative
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, vortex_case, vortex_primitive

    case, _ = vortex_case(40, split=split)
    s = case.numerics
    s.limiter = limiter
    g = build_geometry(case.mesh, case)
    P = vortex_primitive(cell_centroids(case.mesh))
    P *= 1.0 + 0.01 * np.random.default_rng(4).standard_normal(P.shape)
    U0 = torch.as_tensor(primitive_to_conservative(P, s.gamma), device=cuda_device)
    return DeviceGeometry(g), s, U0


def _steps(dg, cfg, U0, scheme, fused, n=4, dt=1e-3):
    dg.set_fused_stage(fused)
    dts = torch.full((1,), dt, dtype=torch.float64, device=U0.device)
    U = U0.clone()
    for _ in range(n):
        dg.explicit_step(U, cfg, scheme, dts)
    dg.check_status()
    dg.set_fused_stage(False)
    return U.cpu().numpy()


@pytest.mark.parametrize("split,limiter", (("half", "Venkatakrishnan"), ("all", "Barth-Jespersen"),
                                           ("half", "Van Leer"), ("all", "Minmod")))
def test_one_launch_stage_equals_launch_per_kernel(cuda_device, split, limiter):
    from meshcfd_gb300.device import make_config

    dg, s, U0 = _vortex(split, limiter, cuda_device)
    cfg = make_config(s, "fast")
    for scheme in (0, 1, 2, 3):  # Euler, RK2, RK3, SSPRK(5,4) (the last falls back)
        np.testing.assert_array_equal(_steps(dg, cfg, U0, scheme, True), _steps(dg, cfg, U0, scheme, False))
    assert dg.fused_stage_blocks >= 1
    dg.close()


def test_one_launch_stage_is_refused_outside_its_settings(cuda_device):
    """The exact variant (and the smooth limiter) keep one launch per kernel
    with the switch on: the results equal the switch off."""
    from meshcfd_gb300.device import make_config

    dg, s, U0 = _vortex("half", "Venkatakrishnan", cuda_device)
    cfg = make_config(s, "exact")
    np.testing.assert_array_equal(_steps(dg, cfg, U0, 2, True), _steps(dg, cfg, U0, 2, False))
    s.limiter, s.venkatakrishnan_k = "Venkatakrishnan K", 5.0
    cfg = make_config(s, "fast")
    np.testing.assert_array_equal(_steps(dg, cfg, U0, 2, True), _steps(dg, cfg, U0, 2, False))
    assert dg.lib.mcfd_set_fused_stage(dg.handle, 2) == 1
    dg.close()


def test_one_launch_stage_batch_with_walls_and_far_field(cuda_device):
    """A batch of uneven channel cases (slip walls, far field), per-cell time
    steps, captured in a CUDA graph: the one-launch stages equal the launch
    per kernel bit for bit."""
    from meshcfd_gb300.batch import BatchStepper, batch_workload, build_batch
    from meshcfd_gb300.device import DeviceGeometry, primitive_to_conservative

    cases = batch_workload(n_cases=6, low=1500, high=6000, seed=5)
    geo, layout, P0, _ = build_batch(cases)
    s = cases[0][0].numerics
    U0 = primitive_to_conservative(P0, s.gamma)
    dg = DeviceGeometry(geo)
    out = []
    for fused in (False, True):
        dg.set_fused_stage(fused)
        stepper = BatchStepper(dg, layout, s, mode="fast")
        U = torch.as_tensor(U0, device=cuda_device)
        stepper.capture(U, 3)  # one eager warm-up step, then 3 captured
        stepper.replay()
        torch.cuda.synchronize()
        dg.check_status()
        out.append(U.cpu().numpy())
    np.testing.assert_array_equal(out[1], out[0])
    dg.close()
