"""Launch shapes (block sizes, faces per thread, and the fast variant's
reconstruction with one thread per cell or one per (cell, variable)) change
no result: residuals and RK3 steps are bit-identical under every shape, and
the autotuner's choice can be replayed with mcfd_set_launch_shapes."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SHAPES = ((0, 0, 0, 0, 0), (0, 0, 0, 0, 1), (64, 128, 2, 64, 1), (256, 64, 4, 128, 1), (128, 256, 1, 256, 0))


@pytest.mark.parametrize("split,limiter", (("half", "Venkatakrishnan"), ("all", "Barth-Jespersen"),
                                           ("half", "Van Leer"), ("half", "Minmod")))
def test_every_launch_shape_gives_the_same_bits(cuda_device, split, limiter):
    from meshcfd_gb300.device import DeviceGeometry, make_config, primitive_to_conservative
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, vortex_case, vortex_primitive

    case, _ = vortex_case(48, split=split)
    s = case.numerics
    s.limiter = limiter
    g = build_geometry(case.mesh, case)
    P = vortex_primitive(cell_centroids(case.mesh))
    P *= 1.0 + 0.01 * np.random.default_rng(9).standard_normal(P.shape)
    U0 = torch.as_tensor(primitive_to_conservative(P, s.gamma), device=cuda_device)
    dg = DeviceGeometry(g)
    cfg = make_config(s, "fast")
    dt = torch.full((1,), 1e-3, dtype=torch.float64, device=cuda_device)
    results = []
    for shape in SHAPES:
        assert dg.lib.mcfd_set_launch_shapes(dg.handle, (C.c_int32 * 5)(*shape)) == 0
        R = dg.residual(U0, cfg).cpu().numpy()
        U = U0.clone()
        for _ in range(3):
            dg.explicit_step(U, cfg, 2, dt)
        results.append((R, U.cpu().numpy()))
    dg.check_status()
    for R, U in results[1:]:
        np.testing.assert_array_equal(R, results[0][0])
        np.testing.assert_array_equal(U, results[0][1])
    chosen = dg.autotune(U0, cfg)
    assert chosen["reconstruct_per_variable"] in (0, 1)
    np.testing.assert_array_equal(dg.residual(U0, cfg).cpu().numpy(), results[0][0])
    assert dg.lib.mcfd_set_launch_shapes(dg.handle, (C.c_int32 * 5)(0, 0, 0, 0, 2)) == 1
