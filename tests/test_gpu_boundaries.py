"""Pressure-inlet and mass-flow boundaries on the GPU against the oracle and
the reference's own outputs.  Their states take libm / NumPy powers (and a
bisection whose last steps turn on last-place differences), so the bar is the
tolerance one: <= 1e-12 relative per residual, not bit-exactness.
"""

import numpy as np
import pytest

from conftest import load_fixture, residual_keys, settings_for, solve_settings

pytestmark = pytest.mark.gpu

FIXTURES = ("bc_pinlet.npz", "bc_massflow.npz")


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("mode", ("exact", "fast"))
@pytest.mark.parametrize("name", FIXTURES)
def test_boundary_residuals_match_oracle_and_reference(cuda_device, name, mode):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from oracle.oracle import Oracle

    data, geom = load_fixture(name)
    dg = DeviceGeometry(geom)
    orc = Oracle(geom)
    U = torch.as_tensor(data["U"], device=cuda_device)
    for key in residual_keys(data):
        s = settings_for(key)
        R = dg.residual(U, make_config(s, mode)).cpu().numpy()
        dg.check_status()
        assert rel_err(R, orc.residual(data["U"], s)) <= 1e-14, key
        assert rel_err(R, data[key]) <= 1e-13, key


@pytest.mark.parametrize("name", FIXTURES)
def test_boundary_time_steps_match_oracle_and_reference(cuda_device, name):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.model import NumericalSettings
    from oracle.oracle import Oracle

    data, geom = load_fixture(name)
    dg = DeviceGeometry(geom)
    s = NumericalSettings(cfl=float(data["cfl"]))
    cfg = make_config(s)
    P = dg.primitive(torch.as_tensor(data["U"], device=cuda_device), cfg)
    dt, dt_min = dg.time_steps(P, cfg, per_cell=True)
    dg.check_status()
    dt = dt.cpu().numpy()
    orc = Oracle(geom)
    assert rel_err(dt, orc.stable_time_steps(orc.primitive(data["U"], 1.4), s)) <= 1e-14
    assert rel_err(dt, data["dt_cells"]) <= 1e-14
    assert float(dt_min) == float(dt.min())


@pytest.mark.parametrize("name", ("solve_pinlet_rk3.npz", "solve_massflow_rk3.npz"))
def test_boundary_solves_match_reference(cuda_device, name):
    import torch
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.solver import run_explicit
    from oracle.oracle import Oracle

    data, geom = load_fixture(name)
    s = solve_settings(data)
    orc = Oracle(geom)
    U0 = orc.conservative(data["P0"], s.gamma)
    U = torch.as_tensor(U0, device=cuda_device)
    result = run_explicit(DeviceGeometry(geom), s, U, final_residual=False)
    P = orc.primitive(U.cpu().numpy(), s.gamma)
    assert rel_err(P, data["P_final"]) <= 1e-12
    assert abs(result.time - float(data["time"])) <= 1e-14 * float(data["time"])


def _channel(kind):
    from make_golden import bc_case

    if kind != "massflow-wide":
        return bc_case(kind)
    # one mass-flow inlet patch of nine faces (the reference's own state
    # function handles one face per patch only)
    case = bc_case("pinlet")
    for c in case.boundary_conditions:
        if c.patch_name == "left":
            c.kind = "Mass Flow Inlet"
            c.values = {"mass_flow": 0.3, "temperature": 1.1 / 287.05, "velocity_x": 1.0, "velocity_y": -0.1}
        elif c.patch_name == "right":
            c.kind = "Mass Flow Outlet"
            c.values = {"mass_flow": 0.3}
    return case


@pytest.mark.parametrize("kind", ("pinlet", "massflow", "massflow-wide"))
def test_boundary_rk3_steps_match_oracle(cuda_device, kind):
    """20 RK3 steps, HLLC + MUSCL-Venkatakrishnan, against the oracle; the
    wide mass-flow inlet is one patch of nine faces (one speed for the patch,
    found on the integrated flow rate)."""
    import torch
    from make_golden import bc_primitive
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.geometry import build_geometry
    from oracle.oracle import Oracle

    case = _channel(kind)
    s = case.numerics
    s.flux, s.reconstruction, s.limiter = "HLLC", "MUSCL linear", "Venkatakrishnan"
    s.time_integration = "Explicit RK3"
    g = build_geometry(case.mesh, case)
    assert len(g.pressure_inlets) + len(g.mass_flow_inlets) > 0
    orc = Oracle(g)
    U0 = orc.conservative(bc_primitive(len(g.areas), seed=5), s.gamma)
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


@pytest.mark.parametrize("kind", ("Pressure Inlet", "Mass Flow Inlet"))
def test_inlet_direction_out_of_domain_raises_the_reference_error(cuda_device, kind):
    """test_solver.py:1063-1079: the message names the patch."""
    import torch
    from make_golden import bc_primitive
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.errors import SolverError
    from meshcfd_gb300.geometry import build_geometry
    from oracle.oracle import Oracle

    case = _channel("pinlet")
    inlet = case.condition("left")
    inlet.kind = kind
    inlet.values = ({"pressure": 1.2, "temperature": 1.1 / 287.05} if kind == "Pressure Inlet"
                    else {"mass_flow": 0.3, "temperature": 1.1 / 287.05})
    inlet.values.update({"velocity_x": -1.0, "velocity_y": 0.0})
    g = build_geometry(case.mesh, case)
    dg = DeviceGeometry(g)
    U = torch.as_tensor(Oracle(g).conservative(bc_primitive(len(g.areas), seed=5), 1.4), device=cuda_device)
    dg.residual(U, make_config(case.numerics))
    with pytest.raises(SolverError, match=r"'left' .*direction must point into the domain"):
        dg.check_status()


def test_pressure_inlet_supersonic_inflow_raises(cuda_device):
    """A face whose interior state flows in supersonically (Mach <= -1):
    "needs Mach number to define a supersonic inflow" (solver.py:4445-4449)."""
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.errors import SolverError
    from meshcfd_gb300.geometry import build_geometry
    from oracle.oracle import Oracle

    case = _channel("pinlet")
    case.numerics.reconstruction = "First order"
    g = build_geometry(case.mesh, case)
    P = np.tile((1.0, 3.0, 0.0, 1.0), (len(g.areas), 1))  # u = 3 > c = 1.18, into the domain
    dg = DeviceGeometry(g)
    U = torch.as_tensor(Oracle(g).conservative(P, 1.4), device=cuda_device)
    dg.residual(U, make_config(case.numerics))
    with pytest.raises(SolverError, match="Pressure inlet 'left' needs Mach number to define a supersonic inflow"):
        dg.check_status()
