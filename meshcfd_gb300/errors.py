"""Error types and messages of the residual/step path.

``SolverError`` mirrors the reference's ``SolverError(ValueError)``
(``src/meshcfd/core/solver.py:50``).  The messages are the reference's own, so
that callers matching on them keep working:

* euler.py:39        "Euler state has non-finite or non-positive density or pressure."
* euler.py:165       "HLLC flux produced a non-finite value."
* euler.py:192       "Roe average has a non-positive sound speed."
* euler.py:261       "Roe flux produced a non-finite value."
* solver.py:2717     "Spatial residual contains non-finite values."
* solver.py:4383     "Far-field characteristics produced invalid sound speed."
* solver.py:4407     "Far-field characteristics produced an invalid state."
* solver.py:4342     "Local stable time steps must be positive and finite."
* solver.py:4424-4566 the pressure-inlet / mass-flow messages, which name the
  boundary patch.
"""

from __future__ import annotations


class SolverError(ValueError):
    """Raised when a case cannot be advanced (mirror of the reference class)."""


# Device status bits (same values as include/meshcfd_gb300.h).
STATUS_NONPHYSICAL_STATE = 1 << 0
STATUS_NONFINITE_RESIDUAL = 1 << 1
STATUS_HLLC_NONFINITE = 1 << 2
STATUS_ROE_SOUND = 1 << 3
STATUS_ROE_NONFINITE = 1 << 4
STATUS_FARFIELD_SOUND = 1 << 5
STATUS_FARFIELD_STATE = 1 << 6
STATUS_TIME_STEP = 1 << 7
STATUS_PIN_DIRECTION = 1 << 8
STATUS_PIN_SUPERSONIC_OUT = 1 << 9
STATUS_PIN_SUPERSONIC_IN = 1 << 10
STATUS_PIN_INCOMPATIBLE = 1 << 11
STATUS_PIN_STATE = 1 << 12
STATUS_MFI_DIRECTION = 1 << 13
STATUS_MFI_PRESSURE = 1 << 14
STATUS_MFI_FLOW_RATE = 1 << 15
STATUS_MFO_DENSITY = 1 << 16
STATUS_VISC_TEMPERATURE = 1 << 17
STATUS_VISC_SUTHERLAND = 1 << 18
STATUS_VISC_DISTANCE = 1 << 19
# no counterpart in the reference: an LU-SGS sweep stopped after a bounded wait
STATUS_SWEEP_TIMEOUT = 1 << 20


class StatusCode(int):
    """Device status bits plus the name of the lowest failing boundary patch
    (``patch``), for the messages that name it."""

    patch = None

# (bit, exception class, message) in the order the reference would raise them
# within one residual evaluation: the state check runs first (inside the
# primitive recovery), flux errors next, the residual finiteness check last.
STATUS_MESSAGES = (
    (STATUS_NONPHYSICAL_STATE, ValueError,
     "Euler state has non-finite or non-positive density or pressure."),
    (STATUS_ROE_SOUND, ValueError, "Roe average has a non-positive sound speed."),
    (STATUS_FARFIELD_SOUND, SolverError,
     "Far-field characteristics produced invalid sound speed."),
    (STATUS_FARFIELD_STATE, SolverError,
     "Far-field characteristics produced an invalid state."),
    (STATUS_PIN_DIRECTION, SolverError,
     "Pressure inlet '{patch}' flow direction must point into the domain across every face."),
    (STATUS_PIN_SUPERSONIC_OUT, SolverError, "Pressure inlet '{patch}' cannot prescribe a supersonic outflow."),
    (STATUS_PIN_SUPERSONIC_IN, SolverError,
     "Pressure inlet '{patch}' needs Mach number to define a supersonic inflow."),
    (STATUS_PIN_INCOMPATIBLE, SolverError,
     "Pressure inlet '{patch}' total conditions are incompatible with the interior characteristic state."),
    (STATUS_PIN_STATE, SolverError, "Pressure inlet '{patch}' produced an invalid state."),
    (STATUS_MFI_DIRECTION, SolverError,
     "Mass-flow inlet '{patch}' direction must point into the domain across every face."),
    (STATUS_MFI_PRESSURE, SolverError, "Mass-flow inlet '{patch}' has invalid interior pressure."),
    (STATUS_MFI_FLOW_RATE, SolverError, "Mass-flow inlet '{patch}' cannot satisfy the configured flow rate."),
    (STATUS_MFO_DENSITY, SolverError, "Mass-flow outlet '{patch}' has invalid interior density."),
    (STATUS_VISC_TEMPERATURE, SolverError, "Viscous flow requires finite positive temperature."),
    (STATUS_VISC_SUTHERLAND, SolverError, "Sutherland law produced an invalid viscosity."),
    (STATUS_VISC_DISTANCE, SolverError, "Boundary face has invalid cell-center distance."),
    (STATUS_HLLC_NONFINITE, ValueError, "HLLC flux produced a non-finite value."),
    (STATUS_ROE_NONFINITE, ValueError, "Roe flux produced a non-finite value."),
    (STATUS_NONFINITE_RESIDUAL, SolverError, "Spatial residual contains non-finite values."),
    (STATUS_TIME_STEP, SolverError, "Local stable time steps must be positive and finite."),
    (STATUS_SWEEP_TIMEOUT, RuntimeError, "LU-SGS sweep waited past its bound for a row it depends on."),
)


def raise_for_status(code: int, solver_error=SolverError) -> None:
    """Raise the reference's exception for the first error bit set in ``code``.

    ``solver_error`` lets a caller substitute its own ``SolverError`` class (the
    drop-in passes the reference's class)."""
    if not code:
        return
    for bit, kind, message in STATUS_MESSAGES:
        if code & bit:
            if "{patch}" in message:
                message = message.format(patch=getattr(code, "patch", None) or "?")
            if kind is SolverError:
                raise solver_error(message)
            raise kind(message)
    raise RuntimeError(f"device reported unknown status 0x{code:x}")
