"""GPU time loop for the explicit integrators, mirroring the reference's
``solve_case`` step loop (solver.py:437-1008) with the state kept in HBM.

Per step: the time step (global adaptive: min over cells and
``end_time - time``; global fixed; local steady: per-cell array and its
mean), one explicit step whose last stage already computes the next step's
time steps from the primitive it recovers, the status words checked
(the stages' with this step, the look-ahead time steps' with the next),
callbacks and convergence history as the reference emits them.  Adaptation
and SST are outside this path.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from time import thread_time

import numpy as np
import torch

from .device import TIME_SCHEME_CODES, DeviceGeometry, make_config
from .errors import SolverError, StatusCode, raise_for_status


@dataclass(frozen=True)
class SolverProgress:
    """Mirror of ``SolverProgress`` (solver.py:57-66)."""

    step: int
    time: float
    time_step: float
    residuals: tuple
    states: object = None
    mesh: object = None
    cpu_time: float = 0.0
    warning: str | None = None


@dataclass(frozen=True)
class SolverResult:
    """Mirror of ``SolverResult`` (solver.py:69-76); ``conservative`` keeps the
    final device state."""

    states: object
    time: float
    steps: int
    residual: float
    completed: bool
    cpu_time: float = 0.0
    conservative: torch.Tensor | None = None


def run_explicit(geom: DeviceGeometry, settings, U: torch.Tensor, *, start_time: float = 0.0,
                 step_offset: int = 0, progress_callback=None, cancel_callback=None,
                 solution_callback=None, solution_interval: int = 1, mode: str = "fast",
                 solver_error=SolverError, check_every: int = 1, final_residual: bool = True):
    """Advance ``U`` (device (C,4) float64, modified in place) like the
    reference's explicit loop.  Returns a :class:`SolverResult`.

    ``mode``: "fast" (the default) keeps exact IEEE arithmetic in the
    reference's operation order and takes each cell's limiter minimum through
    its smallest ratio (three divisions per variable instead of one per
    limiter entry; the same factor for Barth-Jespersen and Minmod, and for the
    smooth limiters unless two candidates round to a last-place tie); "exact"
    evaluates every limiter entry as the reference does; "fma" contracts
    products (outside the 1e-12 bar on fine meshes)."""
    cpu_start = thread_time()
    if settings.time_integration not in TIME_SCHEME_CODES:
        raise NotImplementedError(f"{settings.time_integration} is not an explicit integrator")
    cfg = make_config(settings, mode)
    scheme = TIME_SCHEME_CODES[settings.time_integration]
    local = settings.time_step_mode == "Local (steady)"
    fixed = settings.time_step_mode == "Global fixed"
    dev = geom.device
    # each step's last stage also computes the next step's stable time steps
    # (mcfd_explicit_step_next) into the other buffer of dt_a / dt_b; their
    # status bits are a word of their own, raised by the step that uses them,
    # where the reference computes them (at the top of its loop)
    dt_a = torch.empty(geom.n_cells if local else 1, dtype=torch.float64, device=dev)
    dt_b = torch.empty_like(dt_a)
    ahead = False  # dt_a holds U's time steps and the handle's primitive buffer U's primitive
    # the first stage leaves R(U) in R: the reference's progress report takes
    # the RMS of the residual at the start of the step (solver.py:466, 943-950)
    start_residual = progress_callback is not None and not local
    R = torch.empty_like(U)
    sums = torch.empty(4, dtype=torch.float64, device=dev)
    time = start_time
    steps = step_offset
    completed = False
    derivative_valid = False
    for local_step in range(1, settings.max_iterations + 1):
        step = step_offset + local_step
        if cancel_callback is not None and cancel_callback():
            break
        check = local_step % check_every == 0 or local
        try:
            if ahead:
                code = geom.status_code(look_ahead=True) if check and not fixed else StatusCode(0)
            else:
                P = geom.primitive(U, cfg, out=geom.primitive_buffer())
                if local:
                    cells, _ = geom.time_steps(P, cfg, per_cell=True)
                    dt_a.copy_(cells)
                elif not fixed:
                    geom.time_steps(P, cfg, time_limit=settings.end_time - time, out_min=dt_a)
                code = geom.status_code() if check else StatusCode(0)
            raise_for_status(code, solver_error)
            if fixed:
                time_step = min(settings.fixed_time_step, settings.end_time - time)
                dt_a.fill_(time_step)
            else:
                time_step = float(dt_a.mean()) if local else float(dt_a.item())
            if not math.isfinite(time_step) or time_step <= 0.0:
                raise solver_error("The stable time step is non-positive or non-finite.")
            geom.explicit_step_next(U, cfg, scheme, dt_a, next_dt_cells=dt_b if local else None,
                                    next_dt_min=None if (local or fixed) else dt_b,
                                    time_limit=settings.end_time - (time + time_step), primitive_current=ahead,
                                    start_residual=R if start_residual else None)
            if not fixed:
                dt_a, dt_b = dt_b, dt_a
            ahead = True
            derivative_valid = start_residual
            if check:
                raise_for_status(geom.status_code(), solver_error)
        except (FloatingPointError, ValueError, ZeroDivisionError) as error:
            raise solver_error(f"Solver failed at step {step}: {error}") from error
        time += time_step
        steps = step
        steady_converged = False
        if local:
            geom.residual(U, cfg, out=R)
            derivative_valid = True
            raise_for_status(geom.status_code(), solver_error)
            s = geom.residual_sumsq(R, out=sums)
            steady_residual = math.sqrt(float(s.sum()) / (4 * geom.n_cells))
            steady_converged = steady_residual <= settings.residual_tolerance
        end_time_reached = (not local) and time >= settings.end_time * (1.0 - 1e-13)
        final_step = (end_time_reached or steady_converged or local_step == settings.max_iterations
                      or (cancel_callback is not None and cancel_callback()))
        if progress_callback is not None and (step % settings.convergence_history_interval == 0 or final_step):
            if not derivative_valid:
                geom.residual(U, cfg, out=R)
            s = geom.residual_sumsq(R, out=sums).cpu().numpy()
            rms = tuple(float(v) for v in np.sqrt(s / geom.n_cells))
            progress_callback(SolverProgress(step, time, time_step, rms, None, None, thread_time() - cpu_start))
        if solution_callback is not None and step % solution_interval == 0:
            solution_callback(step, time, U)
        if end_time_reached:
            time = settings.end_time
            completed = True
            break
        if steady_converged:
            completed = True
            break
    # the time steps the last step looked ahead to belong to a step not taken:
    # the reference never computes them, so their bits raise nothing
    geom.status_code(look_ahead=True)
    raise_for_status(geom.status_code(), solver_error)
    residual = float("nan")
    if final_residual:
        geom.residual(U, cfg, out=R)
        raise_for_status(geom.status_code(), solver_error)
        residual = math.sqrt(float(geom.residual_sumsq(R, out=sums).sum()) / (4 * geom.n_cells))
    return SolverResult(None, time, steps, residual, completed, thread_time() - cpu_start, U)
