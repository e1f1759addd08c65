"""Drop-in: put the GPU path behind the reference solver's own calls.

The reference's hot path is a set of module functions of
``meshcfd.core.solver``; its own tests replace them with ``monkeypatch``
(tests/test_solver.py:1300-1306, 802-804).  :func:`install` does the same with
GPU-backed versions taking and returning NumPy arrays:

* ``_residual(conservative, geometry, settings, turbulence=None)``   solver.py:2437
* ``_stable_time_steps(primitive, geometry, settings, turbulence=None)`` solver.py:4132
* ``_stable_time_step(primitive, geometry, settings, turbulence=None)``  solver.py:4117
* ``_explicit_rk4_step(state, time_step, geometry, settings)``          solver.py:1128
* ``_implicit_euler_step(initial, time_step, geometry, settings, ...)``  solver.py:1337

so ``solve_case`` runs unchanged on top of them.  :func:`solve_case` goes
further: after the reference's own checks of the case, it keeps the state in
HBM for the whole explicit loop and returns the reference's ``SolverResult``.  Inviscid and laminar viscous (constant or
Sutherland) cases, first-order, MUSCL-linear and MUSCL-parabolic
reconstruction and every boundary kind of ``_residual`` run on the GPU.
Refused with ``NotImplementedError`` (nothing falls back to the CPU): SST
turbulence states, and in :func:`solve_case` the implicit integrator and
adaptive refinement (use :func:`install` and the reference's own loop for
those).  Walls with a prescribed velocity take their velocities from the
geometry as the reference computed them.
"""

from __future__ import annotations

import weakref

import numpy as np
import torch

from .device import TIME_SCHEME_CODES, DeviceGeometry, make_config
from .errors import raise_for_status

_PATCHED = ("_residual", "_stable_time_steps", "_stable_time_step", "_explicit_rk4_step", "_implicit_euler_step")


class _Cache:
    """DeviceGeometry per reference ``_Geometry`` object (rebuilt after
    adaptation, solver.py:864, so keyed by identity).  Entries go when their
    geometry is collected; geometries that cannot be weakly referenced are
    held strongly, at most ``STRONG_LIMIT`` of them (oldest dropped first)."""

    STRONG_LIMIT = 4

    def __init__(self):
        self.items = {}
        self.strong = []

    def get(self, geometry) -> DeviceGeometry:
        key = id(geometry)
        hit = self.items.get(key)
        if hit is not None and hit[0]() is geometry:
            return hit[1]
        dg = DeviceGeometry(geometry)
        try:
            ref = weakref.ref(geometry, lambda _r, k=key: self.items.pop(k, None))
        except TypeError:
            ref = lambda g=geometry: g  # noqa: E731  (no weakref support: held strongly)
            self.strong.append(key)
            while len(self.strong) > self.STRONG_LIMIT:
                self.items.pop(self.strong.pop(0), None)
        self.items[key] = (ref, dg)
        return dg


_cache = _Cache()


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("meshcfd_gb300 drop-in needs a CUDA device (no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def _solver_error(module):
    return getattr(module, "SolverError", None) if module is not None else None


def make_residual(module=None):
    solver_error = _solver_error(module)

    def _residual(conservative, geometry, settings, turbulence_conservative=None):
        if turbulence_conservative is not None:
            raise NotImplementedError("SST turbulence is not implemented by the GPU residual path")
        dg = _cache.get(geometry)
        cfg = make_config(settings)
        U = torch.as_tensor(np.ascontiguousarray(conservative, dtype=np.float64), device=_device())
        R = dg.residual(U, cfg)
        raise_for_status(dg.status_code(), solver_error or ValueError)
        return R.cpu().numpy()

    return _residual


def make_stable_time_steps(module=None):
    solver_error = _solver_error(module)

    def _stable_time_steps(primitive, geometry, settings, turbulence_conservative=None):
        if turbulence_conservative is not None:
            raise NotImplementedError("SST turbulence is not implemented by the GPU time-step path")
        dg = _cache.get(geometry)
        cfg = make_config(settings)
        P = torch.as_tensor(np.ascontiguousarray(primitive, dtype=np.float64), device=_device())
        dt, _ = dg.time_steps(P, cfg, per_cell=True)
        raise_for_status(dg.status_code(), solver_error or ValueError)
        return dt.cpu().numpy()

    return _stable_time_steps


def make_stable_time_step(module=None):
    steps = make_stable_time_steps(module)

    def _stable_time_step(primitive, geometry, settings, turbulence_conservative=None):
        return float(np.min(steps(primitive, geometry, settings, turbulence_conservative)))

    return _stable_time_step


def make_explicit_rk4_step(module=None):
    solver_error = _solver_error(module)

    def _explicit_rk4_step(state, time_step, geometry, settings):
        if np.shape(state)[1] != 4:
            raise NotImplementedError("SST state is not implemented by the GPU RK4 step")
        dg = _cache.get(geometry)
        cfg = make_config(settings)
        dev = _device()
        U = torch.as_tensor(np.array(state, dtype=np.float64, order="C"), device=dev)
        dt = torch.as_tensor(np.atleast_1d(np.asarray(time_step, dtype=np.float64)), device=dev)
        dg.explicit_step(U, cfg, TIME_SCHEME_CODES["Explicit RK4"], dt)
        raise_for_status(dg.status_code(), solver_error or ValueError)
        return U.cpu().numpy()

    return _explicit_rk4_step


def make_implicit_euler_step(module=None):
    solver_error = _solver_error(module) or ValueError

    def _implicit_euler_step(initial, time_step, geometry, settings, allow_time_step_reduction=True):
        from .implicit import ImplicitEuler

        if np.shape(initial)[1] != 4:
            raise NotImplementedError("SST state is not implemented by the GPU implicit step")
        dg = _cache.get(geometry)
        dev = _device()
        U0 = torch.as_tensor(np.array(initial, dtype=np.float64, order="C"), device=dev)
        dt = torch.as_tensor(np.atleast_1d(np.asarray(time_step, dtype=np.float64)).copy(), device=dev)
        stepper = ImplicitEuler(dg, settings, solver_error=solver_error)
        state, used = stepper.step(U0, dt, allow_time_step_reduction)
        used_np = used.cpu().numpy()
        return state.cpu().numpy(), (float(used_np[0]) if np.ndim(time_step) == 0 else used_np)

    return _implicit_euler_step


def install(module):
    """Patch ``module`` (the reference's ``meshcfd.core.solver``) in place.
    Returns the originals for :func:`uninstall`."""
    originals = {name: getattr(module, name) for name in _PATCHED}
    module._residual = make_residual(module)
    module._stable_time_steps = make_stable_time_steps(module)
    module._stable_time_step = make_stable_time_step(module)
    module._explicit_rk4_step = make_explicit_rk4_step(module)
    module._implicit_euler_step = make_implicit_euler_step(module)
    return originals


def uninstall(module, originals) -> None:
    for name, fn in originals.items():
        setattr(module, name, fn)


class _ChecksPassed(Exception):
    """Raised by the stand-in geometry builder of :func:`_reference_checks`."""


def _reference_checks(module, case, start_time, step_offset, solution_interval) -> None:
    """Run the reference's own checks of the case and settings: the prologue
    of ``solve_case`` (solver.py:193-377), which ends in the geometry build
    (solver.py:379).  For the call, the module's ``_build_geometry`` is a
    stand-in that stops the run there, so each failing check raises the
    reference's own ``SolverError`` with its own message, in its own order."""
    build = module._build_geometry

    def stop(mesh, c):
        raise _ChecksPassed

    module._build_geometry = stop
    try:
        module.solve_case(case, start_time=start_time, step_offset=step_offset,
                          solution_interval=solution_interval)
    except _ChecksPassed:
        pass
    else:
        raise RuntimeError("the reference's solve_case returned before its geometry build")
    finally:
        module._build_geometry = build


def solve_case(module, case, initial_states=None, progress_callback=None, cancel_callback=None,
               start_time: float = 0.0, step_offset: int = 0, solution_callback=None, solution_interval: int = 1):
    """The reference's ``solve_case`` (solver.py:179-1008) for the explicit
    integrators with the state resident in HBM for the whole loop.
    ``module`` is the reference's ``meshcfd.core.solver``: its checks of the
    case and settings, geometry builder, initial conditions and result types
    are used as they are."""
    from .solver import run_explicit

    settings = case.numerics
    _reference_checks(module, case, start_time, step_offset, solution_interval)
    if settings.time_integration not in TIME_SCHEME_CODES:
        raise NotImplementedError("the HBM-resident loop covers the explicit integrators")
    if settings.adaptive_mesh:
        raise NotImplementedError("adaptive refinement is outside the GPU path")
    if settings.turbulence_model != "None":
        raise NotImplementedError("SST turbulence is outside the GPU path")
    geometry = module._build_geometry(case.mesh, case)
    if initial_states is None:
        try:
            initial_states = module.evaluate_initial_conditions(case.mesh, case.initial_conditions)
        except ValueError as error:
            raise module.SolverError(f"Could not evaluate initial conditions: {error}") from error
    if len(initial_states) != len(case.mesh.cells):
        raise module.SolverError("Initial state count must match the mesh cell count.")
    primitive = np.array([(s.density, s.velocity_x, s.velocity_y, s.pressure) for s in initial_states], dtype=float)
    conservative = module.primitive_to_conservative(primitive, settings.gamma)
    try:
        module._primitive_from_conservative(conservative, None, settings.gamma)
    except ValueError as error:
        raise module.SolverError(f"Invalid initial state: {error}") from error
    dg = _cache.get(geometry)
    U = torch.as_tensor(conservative, device=_device())

    def progress(p):
        if progress_callback is not None:
            progress_callback(module.SolverProgress(p.step, p.time, p.time_step, p.residuals, None, None, p.cpu_time))

    def snapshot(step, time, Ud):
        P = module._primitive_from_conservative(Ud.cpu().numpy(), None, settings.gamma)
        solution_callback(step, time, module._states_from_solution(P, None))

    result = run_explicit(dg, settings, U, start_time=start_time, step_offset=step_offset,
                          progress_callback=progress if progress_callback else None,
                          cancel_callback=cancel_callback,
                          solution_callback=snapshot if solution_callback else None,
                          solution_interval=solution_interval, solver_error=module.SolverError)
    final = module._primitive_from_conservative(U.cpu().numpy(), None, settings.gamma)
    states = module._states_from_solution(final, None)
    return module.SolverResult(states, result.time, result.steps, result.residual, result.completed, result.cpu_time)
