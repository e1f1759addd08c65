"""Implicit Euler on the device (solver.py:1185-1567).

The Newton iteration, line search and time-step halving run on the host as in
the reference (a handful of decisions per step); everything per cell — the
full-order residual, the first-order finite-difference Jacobian-vector
product, the LU-SGS preconditioner and the restarted GMRES — runs in the
native library (csrc/mcfd_implicit.cu) on HBM-resident vectors.
"""

from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np
import torch

from . import _lib
from .device import DeviceGeometry, _stream_ptr, make_config
from .errors import SolverError, raise_for_status


def _host(values) -> C.Array:
    return (C.c_double * len(values))(*[float(v) for v in values])


class BudgetExceeded(RuntimeError):
    """The caller's wall-clock deadline passed (checked before each GMRES
    solve); the state is left as it was at the start of the step."""


class ImplicitEuler:
    """Device implicit-Euler stepper for one geometry and settings."""

    # work counters (instance values once counting starts)
    attempts = 0
    newton_iterations = 0
    gmres_iterations = 0
    gmres_calls = 0
    gmres_seconds = 0.0
    deadline = None

    def __init__(self, geom: DeviceGeometry, settings, mode: str = "exact", solver_error=SolverError,
                 deadline: float | None = None):
        """``deadline``: optional ``time.perf_counter()`` value after which the
        next GMRES solve raises :class:`BudgetExceeded` instead of starting.
        ``newton_iterations``, ``gmres_iterations``, ``gmres_calls``,
        ``gmres_seconds`` and ``attempts`` count the work done so far."""
        if settings.implicit_preconditioner != "LU-SGS":
            raise NotImplementedError("the GPU implicit path implements the LU-SGS preconditioner")
        self.geom = geom
        self.settings = settings
        self.cfg = make_config(settings, mode)
        self.lib = geom.lib
        self.solver_error = solver_error
        n = geom.n_cells
        dev = geom.device
        self.rate = torch.empty(n, 4, dtype=torch.float64, device=dev)
        self.cand = torch.empty_like(self.rate)
        self.cand_rate = torch.empty_like(self.rate)
        self.rhs = torch.empty_like(self.rate)
        self.correction = torch.empty_like(self.rate)
        self.gmres_iterations = 0
        self.newton_iterations = 0
        self.gmres_calls = 0
        self.gmres_seconds = 0.0
        self.attempts = 0
        self.deadline = deadline

    # -------------------------------------------------------------- helpers
    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: {self.lib.mcfd_error_string(rc).decode()}")

    def _residual(self, U, out):
        self.geom.residual(U, self.cfg, out=out)
        raise_for_status(self.geom.status_code(), self.solver_error)

    def _equation(self, U, U0, R, dt, per_cell, scales, b=None):
        norms = (C.c_double * 2)()
        self._check(self.lib.mcfd_implicit_equation(
            self.geom.handle, U.data_ptr(), U0.data_ptr(), R.data_ptr(), dt.data_ptr(), per_cell,
            scales, b.data_ptr() if b is not None else None, norms, _stream_ptr()), "mcfd_implicit_equation")
        return norms[0], norms[1]

    def scales(self, state):
        """Per-variable scaling of the Newton iteration (solver.py:1393-1413)."""
        m = (C.c_double * 9)()
        self._check(self.lib.mcfd_implicit_scale_maxima(self.geom.handle, C.byref(self.cfg), state.data_ptr(), m,
                                                        _stream_ptr()), "mcfd_implicit_scale_maxima")
        raise_for_status(self.geom.status_code(), self.solver_error)
        gamma = self.settings.gamma
        rho_scale = max(m[0], 1e-12)
        speed_scale = max(max(m[1], m[2]), m[3], 1e-12)
        scales = [max(m[5 + k], 1e-12) for k in range(4)]
        scales[0] = max(scales[0], rho_scale)
        scales[1] = max(scales[1], rho_scale * speed_scale)
        scales[2] = max(scales[2], rho_scale * speed_scale)
        scales[3] = max(scales[3], rho_scale * speed_scale**2, m[4] / (gamma - 1.0))
        return _host(scales)

    # ---------------------------------------------------------------- solve
    def solve_once(self, initial: torch.Tensor, dt: torch.Tensor) -> torch.Tensor:
        """_implicit_euler_solve_once (solver.py:1371-1486) for a flow-only state."""
        s = self.settings
        err = self.solver_error
        per_cell = int(dt.numel() == self.geom.n_cells and self.geom.n_cells != 1)
        state = initial.clone()
        scales = self.scales(state)
        for _ in range(12):
            self.newton_iterations += 1
            self._residual(state, self.rate)
            eq_norm, upd_norm = self._equation(state, initial, self.rate, dt, per_cell, scales, b=self.rhs)
            if eq_norm <= 1e-9 * max(1.0, upd_norm):
                return state
            self._check(self.lib.mcfd_implicit_prepare(self.geom.handle, C.byref(self.cfg), state.data_ptr(),
                                                       dt.data_ptr(), per_cell, scales, _stream_ptr()),
                        "mcfd_implicit_prepare")
            raise_for_status(self.geom.status_code(), err)
            if self.deadline is not None and time.perf_counter() > self.deadline:
                raise BudgetExceeded("wall-clock budget of the implicit step exceeded")
            iters = C.c_int32(0)
            t0 = time.perf_counter()
            rc = self.lib.mcfd_gmres(self.geom.handle, self.rhs.data_ptr(), self.correction.data_ptr(),
                                     float(s.gmres_tolerance), int(s.gmres_max_iterations),
                                     int(s.gmres_krylov_dimension), C.byref(iters), _stream_ptr())
            self.gmres_seconds += time.perf_counter() - t0
            self.gmres_calls += 1
            self.gmres_iterations += iters.value
            if rc == 6:
                raise err(f"Implicit Euler GMRES did not converge within {s.gmres_max_iterations} iterations "
                          f"(relative tolerance {s.gmres_tolerance:g}).")
            if rc == 7:
                raise err("Implicit Euler GMRES broke down (status -1).")
            self._check(rc, "mcfd_gmres")
            raise_for_status(self.geom.status_code(), err)
            accepted = False
            damping = 1.0
            for _ in range(8):
                self._check(self.lib.mcfd_implicit_candidate(self.geom.handle, state.data_ptr(),
                                                             self.correction.data_ptr(), damping, scales,
                                                             self.cand.data_ptr(), _stream_ptr()),
                            "mcfd_implicit_candidate")
                try:
                    self._residual(self.cand, self.cand_rate)
                    cand_norm, _ = self._equation(self.cand, initial, self.cand_rate, dt, per_cell, scales)
                except (SolverError, ValueError, FloatingPointError):
                    cand_norm = math.inf
                if cand_norm < eq_norm:
                    state.copy_(self.cand)
                    accepted = True
                    break
                damping *= 0.5
            if not accepted:
                raise err("Implicit Euler Newton iteration could not reduce its residual.")
        raise err("Implicit Euler Newton iteration did not converge.")

    def step(self, initial: torch.Tensor, dt: torch.Tensor, allow_time_step_reduction: bool = True):
        """_implicit_euler_step (solver.py:1337-1368): halve the time step on
        failure (12 attempts, or 1 for a fixed step).  Returns (state, dt)."""
        attempted = dt.clone()
        last = None
        attempts = 12 if allow_time_step_reduction else 1
        for _ in range(attempts):
            self.attempts += 1
            try:
                return self.solve_once(initial, attempted), attempted
            except SolverError as error:
                last = error
                attempted.mul_(0.5)
            except ValueError as error:
                if isinstance(error, self.solver_error):
                    last = error
                    attempted.mul_(0.5)
                else:
                    raise
        if not allow_time_step_reduction:
            raise self.solver_error(
                f"Implicit Euler could not converge at the configured fixed time step: {last}") from last
        raise self.solver_error(
            f"Implicit Euler could not converge after reducing the time step 12 times; last failure: {last}") from last


def run_implicit(geom: DeviceGeometry, settings, U: torch.Tensor, *, max_steps=None, mode: str = "exact",
                 solver_error=SolverError, monitor=None):
    """The reference's step loop (solver.py:437-500, 890-905) for Implicit
    Euler in any time-step mode.  ``monitor(step, time, R)`` is called with the
    device residual after each step in local (steady) mode.  Returns
    ``(time, steps, converged)``."""
    cfg = make_config(settings, mode)
    stepper = ImplicitEuler(geom, settings, mode, solver_error)
    local = settings.time_step_mode == "Local (steady)"
    fixed = settings.time_step_mode == "Global fixed"
    dev = geom.device
    time = 0.0
    steps = 0
    R = torch.empty_like(U)
    sums = torch.empty(4, dtype=torch.float64, device=dev)
    limit = settings.max_iterations if max_steps is None else max_steps
    for local_step in range(1, limit + 1):
        try:
            P = geom.primitive(U, cfg, out=geom.primitive_buffer())
            if local:
                dt, _ = geom.time_steps(P, cfg, per_cell=True)
            elif fixed:
                dt = torch.full((1,), min(settings.fixed_time_step, settings.end_time - time), dtype=torch.float64,
                                device=dev)
            else:
                _, dmin = geom.time_steps(P, cfg, time_limit=settings.end_time - time)
                dt = dmin.clone()
            raise_for_status(geom.status_code(), solver_error)
            new_state, used = stepper.step(U, dt, allow_time_step_reduction=not fixed)
            U.copy_(new_state)
            time_step = float(used.mean())
        except (FloatingPointError, ValueError, ZeroDivisionError) as error:
            raise solver_error(f"Solver failed at step {local_step}: {error}") from error
        time += time_step
        steps = local_step
        if local:
            geom.residual(U, cfg, out=R)
            raise_for_status(geom.status_code(), solver_error)
            s = geom.residual_sumsq(R, out=sums).cpu().numpy()
            if monitor is not None:
                monitor(local_step, time, s)
            if math.sqrt(float(s.sum()) / (4 * geom.n_cells)) <= settings.residual_tolerance:
                return time, steps, True
        elif time >= settings.end_time * (1.0 - 1e-13):
            return settings.end_time, steps, True
    return time, steps, False
