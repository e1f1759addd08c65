"""The host logic of the HBM-resident explicit loop (`solver.run_explicit`)
against a scripted stand-in for the device handle: where each status bit is
raised (the reference's step numbers, solver.py:437-811), which residual the
progress report takes (the one at the start of the step, solver.py:466,
943-950), the time-step hand-over from one step's look-ahead to the next,
and the end-time limit."""

import math

import pytest
import torch

from meshcfd_gb300.errors import STATUS_NONPHYSICAL_STATE, STATUS_TIME_STEP, SolverError, StatusCode
from meshcfd_gb300.model import NumericalSettings
from meshcfd_gb300.solver import run_explicit


class FakeGeometry:
    """The DeviceGeometry calls run_explicit makes, on CPU tensors: a step
    adds 1 to U; the stable step is 0.1 (or the end-time limit); status bits
    are planted per step, in the stages' word or the look-ahead word."""

    def __init__(self, n_cells=4, stage_bits=None, ahead_bits=None):
        self.device = torch.device("cpu")
        self.n_cells = n_cells
        self.P = torch.zeros(n_cells, 4, dtype=torch.float64)
        self.stage_bits = dict(stage_bits or {})
        self.ahead_bits = dict(ahead_bits or {})
        self.word = 0
        self.ahead_word = 0
        self.steps = 0
        self.residual_calls = 0
        self.primitive_calls = 0
        self.time_limits = []

    def primitive_buffer(self):
        return self.P

    def primitive(self, U, cfg, out=None):
        self.primitive_calls += 1
        out.copy_(U)
        return out

    def time_steps(self, P, cfg, time_limit=math.inf, per_cell=False, out_min=None):
        if per_cell:
            return torch.full((self.n_cells,), 0.1, dtype=torch.float64), None
        out_min.fill_(min(0.1, time_limit))
        return None, out_min

    def explicit_step_next(self, U, cfg, scheme, dt, *, next_dt_min=None, next_dt_cells=None,
                           time_limit=math.inf, primitive_current=False, start_residual=None):
        self.steps += 1
        if start_residual is not None:
            start_residual.fill_(float(U[0, 0]))  # the residual "of U before the step"
        U.add_(1.0)
        if next_dt_min is not None:
            self.time_limits.append(time_limit)
            next_dt_min.fill_(min(0.1, time_limit))
        if next_dt_cells is not None:
            next_dt_cells.fill_(0.1)
        self.word |= self.stage_bits.get(self.steps, 0)
        self.ahead_word |= self.ahead_bits.get(self.steps, 0)

    def status_code(self, stream=None, *, look_ahead=False):
        if look_ahead:
            code, self.ahead_word = self.ahead_word, 0
        else:
            code, self.word = self.word, 0
        return StatusCode(code)

    def residual(self, U, cfg, out=None):
        self.residual_calls += 1
        out.fill_(float(U[0, 0]))
        return out

    def residual_sumsq(self, R, out=None):
        out.copy_((R * R).sum(dim=0))
        return out


def _settings(**kw):
    s = NumericalSettings()
    s.time_integration = "Explicit RK3"
    s.time_step_mode = "Global adaptive"
    s.end_time, s.max_iterations = 100.0, 5
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def _U(n=4):
    return torch.ones(n, 4, dtype=torch.float64)


def test_a_look_ahead_time_step_error_is_raised_by_the_step_that_uses_it():
    g = FakeGeometry(ahead_bits={2: STATUS_TIME_STEP})
    with pytest.raises(SolverError, match=r"^Solver failed at step 3: Local stable time steps must be positive"):
        run_explicit(g, _settings(), _U())
    assert g.steps == 2


def test_the_last_steps_look_ahead_raises_nothing():
    g = FakeGeometry(ahead_bits={5: STATUS_TIME_STEP})
    result = run_explicit(g, _settings(), _U())
    assert result.steps == 5 and g.steps == 5 and not result.completed


def test_a_stage_error_is_raised_by_its_own_step():
    g = FakeGeometry(stage_bits={2: STATUS_NONPHYSICAL_STATE})
    with pytest.raises(SolverError, match=r"^Solver failed at step 2: Euler state has non-finite"):
        run_explicit(g, _settings(), _U())


def test_the_primitive_is_recovered_once_and_steps_carry_the_time_step():
    g = FakeGeometry()
    result = run_explicit(g, _settings(end_time=0.35), _U(), final_residual=False)
    # 0.1, 0.1, 0.1, then the end-time limit 0.05 from the third step's look-ahead
    assert result.completed and result.steps == 4 and result.time == 0.35
    assert g.primitive_calls == 1
    assert g.time_limits[:3] == [0.35 - 0.1, 0.35 - (0.1 + 0.1), 0.35 - (0.1 + 0.1 + 0.1)]


def test_progress_reports_the_residual_at_the_start_of_each_step():
    g = FakeGeometry()
    reports = []
    run_explicit(g, _settings(convergence_history_interval=2), _U(), progress_callback=reports.append,
                 final_residual=False)
    # U starts at 1 and gains 1 per step: the start of step k holds k
    assert [p.step for p in reports] == [2, 4, 5]
    assert [p.residuals[0] for p in reports] == [2.0, 4.0, 5.0]
    assert g.residual_calls == 0  # the first stage's residual, no extra evaluation


def test_local_steady_progress_reports_the_residual_of_the_new_state():
    g = FakeGeometry()
    reports = []
    run_explicit(g, _settings(time_step_mode="Local (steady)", residual_tolerance=1e-300,
                              convergence_history_interval=1), _U(), progress_callback=reports.append,
                 final_residual=False)
    assert [p.residuals[0] for p in reports] == [2.0, 3.0, 4.0, 5.0, 6.0]
