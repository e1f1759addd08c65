"""mcfd_explicit_step_next: an explicit step whose last stage also leaves
the next step's stable time steps.  Marching with it (each step starting
from the primitive the previous step left) gives the same time steps and
states, bit for bit, as the reference's loop order — primitive, stable time
step, step — through mcfd_primitive / mcfd_time_steps / mcfd_explicit_step:
on the periodic vortex (all four integrators, global and per-cell steps,
every kernel variant), on the Riemann case with walls and far field (whose
time step takes the far-field exterior radius), with a body force, and on a
bump channel with a pressure outlet; and with pressure-inlet patches or
viscous terms, where the time steps come from the time-step pass after the
step, the same values."""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _vortex(n=32):
    from meshcfd_gb300.meshes import cell_centroids, vortex_case, vortex_primitive

    case, _ = vortex_case(n, split="half")
    return case, vortex_primitive(cell_centroids(case.mesh))


def _riemann(n=24):
    from meshcfd_gb300.meshes import riemann_case

    case, P = riemann_case(n)
    s = case.numerics
    s.flux, s.reconstruction, s.limiter = "HLLC", "MUSCL linear", "Venkatakrishnan"
    return case, P


def _bump():
    from meshcfd_gb300.meshes import bump_case

    case, P = bump_case(24, 12)
    s = case.numerics
    s.flux, s.time_integration, s.cfl = "HLLC", "Explicit RK3", 0.5
    return case, P


def _march(dg, cfg, scheme, U0, steps, local, fused, end_time=math.inf):
    """(time steps, final state) of ``steps`` steps in the reference's loop
    order, or with the next step's time steps from each step's last stage."""
    U = U0.clone()
    dev = U.device
    P = dg.primitive_buffer()
    dts = []
    t = 0.0
    if fused:
        dg.primitive(U, cfg, out=P)
        a = torch.empty(dg.n_cells if local else 1, dtype=torch.float64, device=dev)
        b = torch.empty_like(a)
        if local:
            cells, _ = dg.time_steps(P, cfg, per_cell=True)
            a.copy_(cells)
        else:
            dg.time_steps(P, cfg, time_limit=end_time - t, out_min=a)
        for _ in range(steps):
            dts.append(a.cpu().numpy().copy())
            t_next = t + float(a.mean() if local else a.item())
            if local:
                dg.explicit_step_next(U, cfg, scheme, a, next_dt_cells=b, primitive_current=True)
            else:
                dg.explicit_step_next(U, cfg, scheme, a, next_dt_min=b, time_limit=end_time - t_next,
                                      primitive_current=True)
            t = t_next
            a, b = b, a
    else:
        for _ in range(steps):
            dg.primitive(U, cfg, out=P)
            if local:
                dt, _ = dg.time_steps(P, cfg, per_cell=True)
                dt = dt.clone()
            else:
                dt = torch.empty(1, dtype=torch.float64, device=dev)
                dg.time_steps(P, cfg, time_limit=end_time - t, out_min=dt)
            dts.append(dt.cpu().numpy().copy())
            t = t + float(dt.mean() if local else dt.item())
            dg.explicit_step(U, cfg, scheme, dt)
    dg.check_status()
    return np.concatenate([d.ravel() for d in dts]), U.cpu().numpy()


@pytest.mark.parametrize("recipe", ("vortex", "riemann", "bump", "gravity"))
@pytest.mark.parametrize("scheme", (0, 1, 2, 3))
def test_step_next_equals_the_reference_loop_order(cuda_device, recipe, scheme):
    from meshcfd_gb300.device import DeviceGeometry, make_config, primitive_to_conservative
    from meshcfd_gb300.geometry import build_geometry

    case, P = {"vortex": _vortex, "riemann": _riemann, "bump": _bump, "gravity": _vortex}[recipe]()
    s = case.numerics
    if recipe == "gravity":
        s.acceleration_x, s.acceleration_y = 0.3, -0.7
    g = build_geometry(case.mesh, case)
    dg = DeviceGeometry(g)
    U0 = torch.as_tensor(primitive_to_conservative(P, s.gamma), device=cuda_device)
    for mode in ("exact", "fast", "fma"):
        cfg = make_config(s, mode)
        _, dt0 = dg.time_steps(dg.primitive(U0, cfg), cfg)
        for local in (False, True):
            # an end time within the 8 steps on the global path exercises the
            # end-time limit of the last steps
            end = math.inf if local else 5.5 * float(dt0.item())
            a = _march(dg, cfg, scheme, U0, 8, local, False, end)
            b = _march(dg, cfg, scheme, U0, 8, local, True, end)
            np.testing.assert_array_equal(b[0], a[0])
            np.testing.assert_array_equal(b[1], a[1])
    dg.close()


@pytest.mark.parametrize("extra", ("pinlet", "massflow", "noslip", "mixed"))
def test_step_next_with_a_separate_time_step_pass(cuda_device, extra):
    """Settings whose time step needs more than the cell state: the exterior
    states of pressure-inlet and mass-flow patches, the viscous diffusivity
    (no-slip walls with velocity inlet and pressure outlet; a slip wall,
    symmetry, far field and mass-flow outlet).  The step falls back to the
    time-step pass after the step; the same values."""
    from make_golden import bc_case, bc_primitive, viscous_case, viscous_primitive
    from meshcfd_gb300.device import DeviceGeometry, make_config, primitive_to_conservative
    from meshcfd_gb300.geometry import build_geometry

    if extra in ("pinlet", "massflow"):
        case, P = bc_case(extra), None
    else:
        case = viscous_case(extra)
    s = case.numerics
    s.flux, s.reconstruction, s.limiter = "HLLC", "MUSCL linear", "Venkatakrishnan"
    g = build_geometry(case.mesh, case)
    n = len(g.areas)
    P = bc_primitive(n, 5) if extra in ("pinlet", "massflow") else viscous_primitive(extra, n, 5)
    dg = DeviceGeometry(g)
    U0 = torch.as_tensor(primitive_to_conservative(P, s.gamma), device=cuda_device)
    cfg = make_config(s, "exact")
    for local in (False, True):
        a = _march(dg, cfg, 2, U0, 5, local, False)
        b = _march(dg, cfg, 2, U0, 5, local, True)
        np.testing.assert_array_equal(b[0], a[0])
        np.testing.assert_array_equal(b[1], a[1])
    dg.close()


@pytest.mark.parametrize("recipe", ("riemann", "bump"))
@pytest.mark.parametrize("scheme", (0, 1, 2, 3))
def test_step_next_start_residual(cuda_device, recipe, scheme):
    """``start_residual`` receives the residual of the state the step starts
    from, the same bits as mcfd_residual on it, with and without the
    look-ahead time steps; the look-ahead's status word stays clear."""
    from meshcfd_gb300.device import DeviceGeometry, make_config, primitive_to_conservative
    from meshcfd_gb300.geometry import build_geometry

    case, P = {"riemann": _riemann, "bump": _bump}[recipe]()
    s = case.numerics
    dg = DeviceGeometry(build_geometry(case.mesh, case))
    U = torch.as_tensor(primitive_to_conservative(P, s.gamma), device=cuda_device)
    cfg = make_config(s, "fast")
    _, dt = dg.time_steps(dg.primitive(U, cfg), cfg)
    dt = dt.clone()
    R = torch.empty_like(U)
    nxt = torch.empty(1, dtype=torch.float64, device=cuda_device)
    for look_ahead in (True, False, True):
        R0 = dg.residual(U, cfg).clone()
        dg.explicit_step_next(U, cfg, scheme, dt, next_dt_min=nxt if look_ahead else None, start_residual=R,
                              primitive_current=True)
        assert torch.equal(R, R0)
    dg.check_status()
    assert dg.status_code(look_ahead=True) == 0
    dg.close()
