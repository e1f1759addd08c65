"""The implicit-Euler step's host logic (`ImplicitEuler.step`, no GPU):
the reference's time-step halving tests (tests/test_solver.py:786-840)
restated with the nonlinear solve replaced, as the reference's own tests
replace `_implicit_euler_solve_once`."""

import pytest
import torch


def _stepper(solve_once, solver_error=None):
    from meshcfd_gb300.errors import SolverError
    from meshcfd_gb300.implicit import ImplicitEuler

    stepper = object.__new__(ImplicitEuler)  # the host logic only: no device handle
    stepper.solver_error = solver_error or SolverError
    stepper.solve_once = solve_once
    return stepper


def _state():
    return torch.tensor([[1.0, 0.2, -0.1, 2.5]], dtype=torch.float64)


def test_implicit_euler_halves_time_step_until_nonlinear_solve_converges():
    from meshcfd_gb300.errors import SolverError

    attempted = []

    def solve_once(initial, dt):
        attempted.append(float(dt[0]))
        if len(attempted) < 3:
            raise SolverError("nonlinear solve did not converge")
        return initial

    U = _state()
    state, used = _stepper(solve_once).step(U, torch.tensor([0.8], dtype=torch.float64))
    assert attempted == [0.8, 0.4, 0.2]
    assert float(used[0]) == 0.2
    assert state is U


def test_implicit_euler_keeps_a_fixed_time_step_on_nonlinear_failure():
    from meshcfd_gb300.errors import SolverError

    attempted = []

    def solve_once(initial, dt):
        attempted.append(float(dt[0]))
        raise SolverError("nonlinear solve did not converge")

    with pytest.raises(SolverError, match="configured fixed time step"):
        _stepper(solve_once).step(_state(), torch.tensor([0.8], dtype=torch.float64), allow_time_step_reduction=False)
    assert attempted == [0.8]


def test_twelve_halvings_then_the_reference_error():
    from meshcfd_gb300.errors import SolverError

    attempted = []

    def solve_once(initial, dt):
        attempted.append(float(dt[0]))
        raise SolverError("nonlinear solve did not converge")

    with pytest.raises(SolverError, match="after reducing the time step 12 times"):
        _stepper(solve_once).step(_state(), torch.tensor([1.0], dtype=torch.float64))
    assert attempted == [0.5**k for k in range(12)]


def test_the_callers_solver_error_halves_and_other_value_errors_propagate():
    class ReferenceSolverError(ValueError):
        pass

    calls = []

    def flaky(initial, dt):
        calls.append(float(dt[0]))
        if len(calls) == 1:
            raise ReferenceSolverError("nonlinear solve did not converge")
        return initial

    _, used = _stepper(flaky, ReferenceSolverError).step(_state(), torch.tensor([0.5], dtype=torch.float64))
    assert calls == [0.5, 0.25] and float(used[0]) == 0.25

    def broken(initial, dt):
        raise ValueError("Euler state has non-finite or non-positive density or pressure.")

    with pytest.raises(ValueError, match="non-positive density"):
        _stepper(broken, ReferenceSolverError).step(_state(), torch.tensor([0.5], dtype=torch.float64))
