"""Laminar viscous terms on the GPU against the oracle and the reference's own
outputs.  Bar: <= 1e-13 relative per residual and time step against the
reference (Sutherland's power is NumPy's SIMD code there, CUDA pow here;
with constant viscosity the BLAS dot / gemv roundings are written out and
the residuals agree to the last place), <= 1e-12 after the solves."""

import numpy as np
import pytest

from conftest import load_fixture, residual_keys, solve_settings, viscous_settings_for

pytestmark = pytest.mark.gpu

KINDS = ("noslip", "mixed", "periodic")


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("mode", ("exact", "fast"))
@pytest.mark.parametrize("kind", KINDS)
def test_viscous_residuals_match_reference_and_oracle(cuda_device, kind, mode):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from oracle.oracle import Oracle

    data, geom = load_fixture(f"viscous_{kind}.npz")
    dg = DeviceGeometry(geom)
    orc = Oracle(geom)
    U = torch.as_tensor(data["U"], device=cuda_device)
    for key in residual_keys(data):
        s = viscous_settings_for(key, data)
        R = dg.residual(U, make_config(s, mode)).cpu().numpy()
        dg.check_status()
        assert rel_err(R, data[key]) <= 1e-13, key
        assert rel_err(R, orc.residual(data["U"], s)) <= 1e-13, key


@pytest.mark.parametrize("kind", KINDS)
def test_viscous_time_steps_match_reference(cuda_device, kind):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config

    data, geom = load_fixture(f"viscous_{kind}.npz")
    dg = DeviceGeometry(geom)
    for key in residual_keys(data)[:1] + [k for k in residual_keys(data) if k.endswith("Constant")][:1]:
        s = viscous_settings_for(key, data)
        s.cfl = 0.7
        cfg = make_config(s)
        P = dg.primitive(torch.as_tensor(data["U"], device=cuda_device), cfg)
        dt, _ = dg.time_steps(P, cfg, per_cell=True)
        dg.check_status()
        assert rel_err(dt.cpu().numpy(), data[f"dt|{s.viscosity_model}"]) <= 1e-14, key


def test_viscous_solve_matches_reference(cuda_device):
    import torch
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.solver import run_explicit
    from oracle.oracle import Oracle

    data, geom = load_fixture("solve_viscous_noslip_rk3.npz")
    s = solve_settings(data)
    orc = Oracle(geom)
    U = torch.as_tensor(orc.conservative(data["P0"], s.gamma), device=cuda_device)
    result = run_explicit(DeviceGeometry(geom), s, U, final_residual=False)
    assert rel_err(orc.primitive(U.cpu().numpy(), s.gamma), data["P_final"]) <= 1e-12
    assert abs(result.time - float(data["time"])) <= 1e-14 * float(data["time"])


@pytest.mark.parametrize("kind", ("noslip", "mixed"))
def test_viscous_rk3_steps_match_oracle(cuda_device, kind):
    """20 RK3 steps (HLLC, MUSCL-Venkatakrishnan, constant viscosity) on a
    geometry from the project's own builder, against the oracle."""
    import torch
    from make_golden import viscous_case, viscous_primitive
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.geometry import build_geometry
    from oracle.oracle import Oracle

    case = viscous_case(kind)
    s = case.numerics
    s.flux, s.reconstruction, s.limiter, s.time_integration = "HLLC", "MUSCL linear", "Venkatakrishnan", "Explicit RK3"
    g = build_geometry(case.mesh, case)
    orc = Oracle(g)
    U0 = orc.conservative(viscous_primitive(kind, len(g.areas), 5), s.gamma)
    dt = 0.5 * float(orc.stable_time_steps(orc.primitive(U0, s.gamma), s).min())
    dg = DeviceGeometry(g)
    cfg = make_config(s)
    U = torch.as_tensor(U0, device=cuda_device)
    dt_dev = torch.full((1,), dt, dtype=torch.float64, device=cuda_device)
    Uo = U0
    for _ in range(20):
        dg.explicit_step(U, cfg, 2, dt_dev)
        Uo = orc.explicit_step(Uo, s, dt)
    dg.check_status()
    assert rel_err(U.cpu().numpy(), Uo) <= 1e-12


def test_viscous_settings_need_the_wall_thermal_data(cuda_device):
    """A geometry built for inviscid flow has no wall thermal data: the viscous
    path refuses it instead of guessing."""
    import torch
    from make_golden import viscous_case
    from meshcfd_gb300._lib import NativeError
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.geometry import build_geometry

    case = viscous_case("noslip")
    case.numerics.viscosity_model = "Inviscid"
    g = build_geometry(case.mesh, case)
    dg = DeviceGeometry(g)
    s = case.numerics
    s.viscosity_model = "Constant"
    U = torch.ones(dg.n_cells, 4, dtype=torch.float64, device=cuda_device) * torch.tensor(
        [1.0, 0.1, 0.0, 3.0], dtype=torch.float64, device=cuda_device)
    with pytest.raises(NativeError, match="not supported"):
        dg.residual(U, make_config(s))
