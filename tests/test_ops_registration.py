"""The PyTorch custom ops over the C ABI (host side, no GPU): registered
under torch.ops.meshcfd_gb300, shapes from their fake implementations on
meta tensors, and CPU tensors refused (there is no CPU path)."""

import pytest
import torch


def _ops():
    import meshcfd_gb300.ops  # noqa: F401  (registers the ops)

    return torch.ops.meshcfd_gb300


def test_ops_are_registered_with_their_schemas():
    ops = _ops()
    for name in ("primitive", "residual", "time_step", "local_time_steps", "explicit_step_"):
        assert hasattr(ops, name), name
    first = ops.explicit_step_.default._schema.arguments[0]
    assert first.name == "U" and first.alias_info is not None and first.alias_info.is_write  # in place


def test_fake_implementations_give_the_output_shapes():
    ops = _ops()
    U = torch.empty(7, 4, dtype=torch.float64, device="meta")
    assert ops.primitive(U, 0, 1.4).shape == (7, 4)
    assert ops.residual(U, 0, 1, 1, 3, 1.4, 0.0, 0.0).shape == (7, 4)
    assert ops.time_step(U, 0, 1.4, 0.8, 1.0).shape == (1,)
    assert ops.local_time_steps(U, 0, 1.4, 0.8).shape == (7,)
    assert ops.explicit_step_(U, torch.empty(1, dtype=torch.float64, device="meta"), 0, 2, 1, 1, 3, 1.4, 0.0,
                              0.0) is None


def test_cpu_tensors_are_refused():
    ops = _ops()
    U = torch.ones(7, 4, dtype=torch.float64)
    with pytest.raises(ValueError, match="no CPU path"):
        ops.residual(U, 0, 1, 1, 3, 1.4, 0.0, 0.0)
    with pytest.raises(ValueError, match="no CPU path"):
        ops.explicit_step_(U, torch.ones(1, dtype=torch.float64), 0, 2, 1, 1, 3, 1.4, 0.0, 0.0)
