"""The FP64 PyTorch-op residual (the autograd cross-check of the reverse
mode) against the reference's own residuals in the golden fixtures."""

import numpy as np
import pytest

from conftest import load_fixture, residual_keys, settings_for

torch = pytest.importorskip("torch")

FIXTURES = ("residual_riemann16.npz", "residual_periodic_mixed.npz", "residual_channel.npz")


@pytest.mark.parametrize("name", FIXTURES)
def test_torch_residual_matches_reference(name):
    from oracle.torch_residual import TorchResidual

    data, geom = load_fixture(name)
    U = torch.as_tensor(data["U"])
    for key in residual_keys(data):
        R = TorchResidual(geom, settings_for(key))(U).numpy()
        ref = data[key]
        assert np.abs(R - ref).max() <= 1e-12 * np.abs(ref).max(), key


def test_torch_residual_far_field_is_differentiable():
    """Gradients reach the far-field states (the adjoint's inflow parameters)
    and agree with central differences on a state away from switches."""
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import riemann_case, smooth_primitive
    from oracle.oracle import Oracle
    from oracle.torch_residual import TorchResidual

    case, _ = riemann_case(8)
    g = build_geometry(case.mesh, case)
    P = smooth_primitive(len(case.mesh.cells), seed=3, amplitude=1.0)
    U = torch.as_tensor(Oracle(g).conservative(P, 1.4))
    s = case.numerics
    s.flux, s.reconstruction, s.limiter = "HLLC", "MUSCL linear", "Venkatakrishnan"
    res = TorchResidual(g, s)
    far = res.far_states.clone().requires_grad_(True)
    lam = torch.as_tensor(np.random.default_rng(0).standard_normal(U.shape))
    (lam * res(U, far)).sum().backward()
    d = torch.as_tensor(np.random.default_rng(1).standard_normal(far.shape))
    h = 1e-6
    with torch.no_grad():
        fd = ((lam * res(U, far + h * d)).sum() - (lam * res(U, far - h * d)).sum()) / (2 * h)
    an = (far.grad * d).sum()
    assert abs(float(fd - an)) <= 1e-6 * max(1.0, abs(float(fd)))
