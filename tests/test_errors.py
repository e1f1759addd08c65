"""Device status words to the reference's exceptions (host logic, no GPU):
the Python bits equal the C ABI's MCFD_S_* values, each bit raises the
reference's class and message, and several bits raise the one the reference
would raise first."""

import re

import pytest

from conftest import ROOT


def _header_bits():
    text = (ROOT / "include" / "meshcfd_gb300.h").read_text()
    return {name: int(value, 16) for name, value in re.findall(r"#define MCFD_S_(\w+) (0x[0-9a-fA-F]+)", text)}


def test_status_bits_equal_the_c_abi():
    from meshcfd_gb300 import errors

    bits = _header_bits()
    assert len(bits) == 21
    for name, value in bits.items():
        assert getattr(errors, "STATUS_" + name) == value, name
    assert sorted(bit for bit, _, _ in errors.STATUS_MESSAGES) == sorted(bits.values())


@pytest.mark.parametrize("index", range(21))
def test_each_bit_raises_the_reference_exception(index):
    from meshcfd_gb300 import errors

    bit, kind, message = errors.STATUS_MESSAGES[index]
    code = errors.StatusCode(bit)
    code.patch = "inlet-a"
    with pytest.raises(kind) as raised:
        errors.raise_for_status(code)
    assert type(raised.value) is kind
    assert str(raised.value) == message.replace("{patch}", "inlet-a")


def test_first_error_in_the_reference_order_wins_and_solver_error_is_substitutable():
    from meshcfd_gb300 import errors

    class ReferenceSolverError(ValueError):
        pass

    both = errors.STATUS_NONFINITE_RESIDUAL | errors.STATUS_NONPHYSICAL_STATE
    with pytest.raises(ValueError, match="non-finite or non-positive density or pressure"):
        errors.raise_for_status(both, ReferenceSolverError)
    with pytest.raises(ReferenceSolverError, match="Spatial residual contains non-finite values"):
        errors.raise_for_status(errors.STATUS_NONFINITE_RESIDUAL | errors.STATUS_TIME_STEP, ReferenceSolverError)
    errors.raise_for_status(0)
    with pytest.raises(RuntimeError, match="unknown status"):
        errors.raise_for_status(1 << 30)
