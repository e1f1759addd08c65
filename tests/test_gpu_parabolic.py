"""MUSCL-parabolic reconstruction on the GPU: bit-exact against the oracle
(same elimination and rank gate, same operation order) and within rounding of
the reference's own LAPACK-based outputs in the golden fixtures.  Far-field
meshes differ from the oracle in the last place of the ghost state's pow().
"""

import numpy as np
import pytest

from conftest import load_fixture, residual_keys, settings_for, solve_settings

pytestmark = pytest.mark.gpu

FIXTURES = ("parabolic_riemann16.npz", "parabolic_periodic_mixed.npz", "parabolic_channel.npz",
            "parabolic_strip.npz")
LIMITERS = ("Barth-Jespersen", "Minmod", "Van Leer", "Venkatakrishnan")
TOL_REFERENCE = 1e-13


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("mode", ("exact", "fast"))
@pytest.mark.parametrize("name", FIXTURES)
def test_parabolic_residual_matches_oracle_and_reference(cuda_device, name, mode):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from oracle.oracle import Oracle

    data, geom = load_fixture(name)
    dg = DeviceGeometry(geom)
    orc = Oracle(geom)
    U = torch.as_tensor(data["U"], device=cuda_device)
    far = len(geom.far_field_faces) > 0
    for key in residual_keys(data):
        s = settings_for(key)
        R = dg.residual(U, make_config(s, mode)).cpu().numpy()
        dg.check_status()
        R_orc = orc.residual(data["U"], s)
        if far:
            assert rel_err(R, R_orc) <= 1e-15, key
        else:
            np.testing.assert_array_equal(R, R_orc, err_msg=key)
        assert rel_err(R, data[key]) <= TOL_REFERENCE, key


@pytest.mark.parametrize("name", FIXTURES)
def test_parabolic_fields_match_oracle_and_reference(cuda_device, name):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.model import NumericalSettings
    from oracle.oracle import Oracle

    data, geom = load_fixture(name)
    dg = DeviceGeometry(geom)
    orc = Oracle(geom)
    P = orc.primitive(data["U"], 1.4)
    Pd = torch.as_tensor(P, device=cuda_device)
    for code, limiter in enumerate(LIMITERS):
        cfg = make_config(NumericalSettings(reconstruction="MUSCL parabolic", limiter=limiter))
        g, k, f = (t.cpu().numpy() for t in dg.reconstruction(Pd, cfg))
        go, ko, fo = orc.parabolic_reconstruction(P, limiter)
        np.testing.assert_array_equal(g, go)
        np.testing.assert_array_equal(k, ko)
        np.testing.assert_array_equal(f, fo)
        assert rel_err(g, data[f"pgrad|{code}"]) <= TOL_REFERENCE
        assert rel_err(k, data[f"pcurv|{code}"]) <= TOL_REFERENCE
        assert rel_err(f, data[f"pfactors|{code}"]) <= TOL_REFERENCE


@pytest.mark.parametrize("name", ("residual_riemann16.npz", "residual_periodic_mixed.npz", "residual_channel.npz"))
def test_linear_fields_match_reference_bit_for_bit(cuda_device, name):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.model import NumericalSettings
    from oracle.oracle import Oracle

    data, geom = load_fixture(name)
    dg = DeviceGeometry(geom)
    P = torch.as_tensor(Oracle(geom).primitive(data["U"], 1.4), device=cuda_device)
    for code, limiter in enumerate(LIMITERS):
        grad, curv, fac = dg.reconstruction(P, make_config(NumericalSettings(limiter=limiter)))
        assert curv is None
        np.testing.assert_array_equal(grad.cpu().numpy(), data[f"grad|{code}"])
        np.testing.assert_array_equal(fac.cpu().numpy(), data[f"factors|{code}"])


def test_parabolic_solve_matches_reference_golden(cuda_device):
    import torch
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.solver import run_explicit
    from oracle.oracle import Oracle

    data, geom = load_fixture("solve_vortex12_rk3_parabolic.npz")
    s = solve_settings(data)
    orc = Oracle(geom)
    U0 = orc.conservative(data["P0"], s.gamma)
    U = torch.as_tensor(U0, device=cuda_device)
    result = run_explicit(DeviceGeometry(geom), s, U, final_residual=False)
    U_orc, t_orc = orc.solve(U0, s, int(data["steps"]))
    np.testing.assert_array_equal(U.cpu().numpy(), U_orc)
    assert result.time == t_orc
    assert rel_err(orc.primitive(U.cpu().numpy(), s.gamma), data["P_final"]) <= 1e-12


@pytest.mark.parametrize("flux", ("Rusanov", "HLLC", "Roe"))
def test_parabolic_rk3_steps_match_oracle_seeded(cuda_device, flux):
    """A larger jittered mixed periodic mesh (the vortex), 20 RK3 steps,
    bit for bit."""
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, vortex_case, vortex_primitive
    from oracle.oracle import Oracle

    case, _ = vortex_case(32, split="half")
    s = case.numerics
    s.flux, s.reconstruction, s.limiter, s.time_integration = flux, "MUSCL parabolic", "Venkatakrishnan", "Explicit RK3"
    g = build_geometry(case.mesh, case)
    assert len(g.parabolic_sources) > 0
    orc = Oracle(g)
    U0 = orc.conservative(vortex_primitive(cell_centroids(case.mesh)), s.gamma)
    dt = 0.5 * float(orc.stable_time_steps(orc.primitive(U0, s.gamma), s).min())
    dg = DeviceGeometry(g)
    U = torch.as_tensor(U0, device=cuda_device)
    dt_dev = torch.full((1,), dt, dtype=torch.float64, device=cuda_device)
    cfg = make_config(s)
    Uo = U0
    for _ in range(20):
        dg.explicit_step(U, cfg, 2, dt_dev)
        Uo = orc.explicit_step(Uo, s, dt)
    dg.check_status()
    np.testing.assert_array_equal(U.cpu().numpy(), Uo)


def test_parabolic_reconstruction_recovers_quadratic_field_on_gpu(cuda_device):
    """test_solver.py:843-872 on the GPU (geometry built with the stencil)."""
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import periodic_case

    case = periodic_case(6, 6)
    case.numerics.reconstruction = "MUSCL parabolic"
    g = build_geometry(case.mesh, case)
    x, y = np.asarray(g.centers).T
    P = np.column_stack((10.0 + x * x + 2.0 * x * y + 3.0 * y * y, np.full_like(x, 0.2), np.full_like(x, -0.1),
                         np.ones_like(x)))
    grad, curv, fac = DeviceGeometry(g).reconstruction(torch.as_tensor(P, device=cuda_device),
                                                       make_config(case.numerics))
    grad, curv, fac = grad.cpu().numpy(), curv.cpu().numpy(), fac.cpu().numpy()
    c = 3 * 6 + 3
    np.testing.assert_allclose(grad[c, 0], (2.0 * x[c] + 2.0 * y[c], 2.0 * x[c] + 6.0 * y[c]), rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(curv[c, 0], (2.0, 2.0, 6.0), rtol=1e-10, atol=1e-10)
    assert fac[c, 0] == pytest.approx(1.0)
