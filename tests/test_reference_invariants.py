"""The reference's own known-answer tests of the explicit path
(tests/test_solver.py:647-732, 1464-1530), restated on each implementation
separately: the oracle on the CPU and the device path on the GPU.  The
invariants follow from the finite-volume scheme, so each side must satisfy
them on its own, with the reference's tolerances."""

import math

import numpy as np
import pytest

FLUXES = ("Rusanov", "HLLC", "Roe")
INTEGRATORS = ("Explicit Euler", "Explicit RK2", "Explicit RK3", "Explicit RK4")
BACKENDS = ("oracle", pytest.param("device", marks=pytest.mark.gpu))


def _march(backend, request, case, settings, P0):
    """The explicit loop from primitive state ``P0`` to ``settings.end_time``;
    returns (initial U, final U, final time, steps)."""
    from meshcfd_gb300.geometry import build_geometry
    from oracle.oracle import Oracle

    g = build_geometry(case.mesh, case)
    orc = Oracle(g)
    U0 = orc.conservative(np.asarray(P0, dtype=np.float64), settings.gamma)
    if backend == "oracle":
        U, t, steps = U0, 0.0, 0
        while t < settings.end_time * (1.0 - 1e-13) and steps < settings.max_iterations:
            U, t = orc.solve(U, settings, 1, time=t)
            steps += 1
        return U0, U, t, steps
    import torch
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.solver import run_explicit

    device = request.getfixturevalue("cuda_device")
    dg = DeviceGeometry(g)
    U = torch.as_tensor(U0, device=device)
    result = run_explicit(dg, settings, U, final_residual=False)
    return U0, U.cpu().numpy(), result.time, result.steps


# the reference's one-cell mesh on the oracle; the device path on the 4 x 3
# mesh (its single-cell, interior-face-free geometry has not run on a GPU)
UNIFORM_MESHES = (("oracle", (1, 1)), ("oracle", (4, 3)), pytest.param("device", (4, 3), marks=pytest.mark.gpu))


@pytest.mark.parametrize("backend,cells", UNIFORM_MESHES)
@pytest.mark.parametrize("flux", FLUXES)
@pytest.mark.parametrize("integrator", INTEGRATORS)
def test_uniform_periodic_flow_is_preserved(backend, request, cells, flux, integrator):
    """test_solver.py:647-679: a uniform state on a periodic mesh (the
    reference uses one cell, its own neighbour across both pairs) stays
    uniform to 1e-12 up to t = 0.9 at CFL 0.5."""
    from meshcfd_gb300.meshes import periodic_case

    case = periodic_case(*cells)
    s = case.numerics
    s.flux, s.time_integration, s.end_time, s.cfl = flux, integrator, 0.9, 0.5
    s.max_iterations, s.residual_tolerance = 10000, 1e-300
    state = (1.0, 0.2, -0.1, 1.0)
    P0 = np.tile(state, (cells[0] * cells[1], 1))
    _, U, t, steps = _march(backend, request, case, s, P0)
    assert steps > 1
    assert abs(t - 0.9) <= 1e-12
    P = _primitive(U, s.gamma)
    np.testing.assert_allclose(P, np.tile(state, (len(P), 1)), rtol=1e-12, atol=1e-12)


def _boundary_case(cells, kinds):
    """The box of ``cells`` with its bottom / right / top / left patches set
    to ``kinds`` (kind, values) and no periodic pairs."""
    from meshcfd_gb300.meshes import box_mesh
    from meshcfd_gb300.model import Case

    case = Case(name="box", mesh=box_mesh(*cells))
    for condition, (kind, values) in zip(case.boundary_conditions, kinds):
        condition.kind, condition.values = kind, dict(values)
    s = case.numerics
    s.gas_constant, s.end_time, s.max_iterations, s.residual_tolerance = 1.0, 0.01, 10000, 1e-300
    return case


INLET = ("Velocity Inlet", {"density": 1.0, "velocity_x": 1.0, "velocity_y": 0.0, "temperature": 1.0})
WALL = ("Wall", {})


@pytest.mark.parametrize("backend,cells", UNIFORM_MESHES)
@pytest.mark.parametrize("flux", FLUXES)
def test_velocity_inlet_and_pressure_outlet_preserve_matching_uniform_flow(backend, request, cells, flux):
    """test_solver.py:877-908: walls below and above, a pressure outlet
    (p = 1) on the right and a velocity inlet (rho = 1, u = 1, R T = 1) on
    the left keep the matching uniform state to 1e-12 up to t = 0.01."""
    case = _boundary_case(cells, (WALL, ("Pressure Outlet", {"pressure": 1.0}), WALL, INLET))
    case.numerics.flux = flux
    state = (1.0, 1.0, 0.0, 1.0)
    _, U, _, _ = _march(backend, request, case, case.numerics, np.tile(state, (cells[0] * cells[1], 1)))
    np.testing.assert_allclose(_primitive(U, 1.4), np.tile(state, (len(U), 1)), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("backend,cells", UNIFORM_MESHES)
def test_pressure_outlet_applies_configured_static_pressure(backend, request, cells):
    """test_solver.py:911-931: a fluid at rest (p = 1) next to an outlet at
    p = 0.8 starts to move towards it in the first step."""
    case = _boundary_case(cells, (WALL, ("Pressure Outlet", {"pressure": 0.8}), WALL,
                                  ("Velocity Inlet", {"density": 1.0, "velocity_x": 0.0, "velocity_y": 0.0,
                                                      "temperature": 1.0})))
    case.numerics.max_iterations = 1
    _, U, _, steps = _march(backend, request, case, case.numerics, np.tile((1.0, 0.0, 0.0, 1.0),
                                                                           (cells[0] * cells[1], 1)))
    assert steps == 1
    nx, ny = cells
    outlet_column = _primitive(U, 1.4)[nx - 1::nx, 1]  # the cells along the right boundary
    assert len(outlet_column) == ny and (outlet_column > 0.0).all()


@pytest.mark.parametrize("backend,cells", UNIFORM_MESHES)
@pytest.mark.parametrize("flux", FLUXES)
def test_far_field_preserves_matching_uniform_flow(backend, request, cells, flux):
    """test_solver.py:1119-1146: far field on every side with the interior's
    uniform state keeps it to 1e-12 up to t = 0.01."""
    far = ("Far Field", {"density": 1.0, "velocity_x": 0.2, "velocity_y": -0.1, "pressure": 1.0})
    case = _boundary_case(cells, (far, far, far, far))
    case.numerics.flux = flux
    state = (1.0, 0.2, -0.1, 1.0)
    _, U, _, _ = _march(backend, request, case, case.numerics, np.tile(state, (cells[0] * cells[1], 1)))
    np.testing.assert_allclose(_primitive(U, 1.4), np.tile(state, (len(U), 1)), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("backend", BACKENDS)
@pytest.mark.parametrize("flux", FLUXES)
@pytest.mark.parametrize("integrator", INTEGRATORS)
@pytest.mark.parametrize("reconstruction", ("First order", "MUSCL linear", "MUSCL parabolic"))
def test_periodic_solver_conserves_integrated_state(backend, request, flux, integrator, reconstruction):
    """test_solver.py:682-732: on the periodic 4 x 3 mesh (equal cells) the
    sum of the conservative states is unchanged to 1e-11 at t = 0.01."""
    from meshcfd_gb300.meshes import periodic_case

    case = periodic_case(4, 3)
    s = case.numerics
    s.flux, s.time_integration, s.reconstruction, s.end_time = flux, integrator, reconstruction, 0.01
    s.max_iterations, s.residual_tolerance = 10000, 1e-300
    P0 = np.array([(1.0 + 0.03 * math.sin(2 * math.pi * (i + 0.5) / 4), 0.2, -0.1,
                    1.0 + 0.02 * math.cos(2 * math.pi * (j + 0.5) / 3)) for j in range(3) for i in range(4)])
    U0, U, t, _ = _march(backend, request, case, s, P0)
    assert abs(t - 0.01) <= 1e-14
    np.testing.assert_allclose(U.sum(axis=0), U0.sum(axis=0), rtol=1e-11, atol=1e-11)


@pytest.mark.parametrize("backend", BACKENDS)
@pytest.mark.parametrize("reconstruction", ("MUSCL linear", "MUSCL parabolic"))
def test_isentropic_vortex_returns_after_one_period(backend, request, reconstruction):
    """test_solver.py:1464-1530: the isentropic vortex (strength 5, free
    stream (1, 1)) on the periodic 10 x 10 mesh of [0, 10]^2, HLLC, RK3,
    Barth-Jespersen, CFL 0.4, advected for one period (t = 10): positive
    density and pressure everywhere and a relative L2 density error < 0.2."""
    from meshcfd_gb300.meshes import cell_centroids, periodic_case

    gamma, beta = 1.4, 5.0
    case = periodic_case(10, 10, 10.0, 10.0)
    s = case.numerics
    s.flux, s.time_integration, s.reconstruction, s.limiter = "HLLC", "Explicit RK3", reconstruction, "Barth-Jespersen"
    s.cfl, s.end_time, s.max_iterations, s.residual_tolerance = 0.4, 10.0, 5000, 1e-300
    xy = cell_centroids(case.mesh)
    dx, dy = xy[:, 0] - 5.0, xy[:, 1] - 5.0
    r2 = dx * dx + dy * dy
    bump = np.exp(0.5 * (1.0 - r2))
    T = 1.0 - (gamma - 1.0) * beta**2 / (8.0 * gamma * math.pi**2) * np.exp(1.0 - r2)
    rho = T ** (1.0 / (gamma - 1.0))
    P0 = np.column_stack((rho, 1.0 - beta / (2 * math.pi) * bump * dy, 1.0 + beta / (2 * math.pi) * bump * dx,
                          rho**gamma))
    _, U, t, steps = _march(backend, request, case, s, P0)
    assert steps < s.max_iterations and abs(t - 10.0) <= 1e-12
    P = _primitive(U, gamma)
    assert (P[:, 0] > 0.0).all() and (P[:, 3] > 0.0).all()
    assert np.linalg.norm(P[:, 0] - rho) / np.linalg.norm(rho) < 0.2


def _primitive(U, gamma):
    rho = U[:, 0]
    u, v = U[:, 1] / rho, U[:, 2] / rho
    return np.column_stack((rho, u, v, (gamma - 1.0) * (U[:, 3] - 0.5 * rho * (u * u + v * v))))
