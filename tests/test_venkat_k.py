"""Venkatakrishnan's limiter with the smoothing constant K (an extension with
no counterpart in the reference, whose Venkatakrishnan form has no K): the
oracle's C restatement of the published formula against the torch-op
residual, and the properties that make it the limiter for gradient checks."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _case(n=10, k=5.0, flux="HLLC"):
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import periodic_case, smooth_primitive

    case = periodic_case(n, n - 2, split="half", jitter=0.2, seed=5)
    s = case.numerics
    s.flux, s.reconstruction, s.limiter = flux, "MUSCL linear", "Venkatakrishnan K"
    s.venkatakrishnan_k = k
    g = build_geometry(case.mesh, case)
    return s, g, smooth_primitive(len(g.areas), seed=3, amplitude=0.2)


@pytest.mark.parametrize("flux", ("Rusanov", "HLLC", "Roe"))
def test_oracle_and_torch_residual_agree(flux):
    from oracle.oracle import Oracle
    from oracle.torch_residual import TorchResidual

    s, g, P = _case(flux=flux)
    orc = Oracle(g)
    U = orc.conservative(P, s.gamma)
    R = orc.residual(U, s)
    Rt = TorchResidual(g, s)(torch.as_tensor(U)).numpy()
    assert np.abs(R - Rt).max() <= 1e-12 * np.abs(R).max()


def test_factors_uniform_state_and_large_k():
    """A uniform state gives factor 1 exactly; as K grows the factor tends to
    1 (the smoothing term dominates); it is not capped at 1."""
    from oracle.oracle import Oracle

    s, g, P = _case()
    orc = Oracle(g)
    _, fac = orc.gradients_and_factors(np.tile(P[0], (len(P), 1)), "Venkatakrishnan K", 5.0)
    assert np.all(fac == 1.0)
    _, f5 = orc.gradients_and_factors(P, "Venkatakrishnan K", 5.0)
    _, f500 = orc.gradients_and_factors(P, "Venkatakrishnan K", 500.0)
    assert np.abs(f500 - 1.0).max() < np.abs(f5 - 1.0).max() and np.abs(f500 - 1.0).max() < 1e-3
    assert f5.max() > 1.0  # the published form exceeds 1 where increments are small against the extrema


def test_residual_is_smooth_where_checked():
    """Torch autograd of the K-form residual against central differences of
    the oracle's residual (h = 1e-7 relative) in a random direction: the
    limiter differentiable, unlike the reference's capped form."""
    from oracle.oracle import Oracle
    from oracle.torch_residual import TorchResidual

    s, g, P = _case()
    orc = Oracle(g)
    U0 = orc.conservative(P, s.gamma)
    rng = np.random.default_rng(4)
    v = rng.standard_normal(U0.shape) * np.abs(U0)
    lam = rng.standard_normal(U0.shape)
    Ut = torch.as_tensor(U0).requires_grad_(True)
    (torch.as_tensor(lam) * TorchResidual(g, s)(Ut)).sum().backward()
    an = float((Ut.grad.numpy() * v).sum())
    h = 1e-7
    fd = float((lam * (orc.residual(U0 + h * v, s) - orc.residual(U0 - h * v, s))).sum()) / (2 * h)
    assert abs(fd - an) <= 1e-6 * abs(fd), (fd, an)
