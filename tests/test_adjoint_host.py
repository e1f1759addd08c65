"""Host pieces of the adjoint (no GPU): the chain rule from primitive
initial states, (dU/dP)^T lambda, against central differences of
primitive_to_conservative (euler.py:8-17)."""

import numpy as np


def test_conservative_jacobian_transpose_matches_central_differences():
    from meshcfd_gb300.adjoint import conservative_jacobian_T
    from meshcfd_gb300.device import primitive_to_conservative

    rng = np.random.default_rng(4)
    n, gamma, h = 50, 1.4, 1e-6
    P = np.column_stack((rng.uniform(0.5, 2.0, n), rng.uniform(-1.0, 1.0, n), rng.uniform(-1.0, 1.0, n),
                         rng.uniform(0.5, 2.0, n)))
    lam = rng.standard_normal((n, 4))
    got = conservative_jacobian_T(P, lam, gamma)
    fd = np.empty_like(P)
    for k in range(4):
        dP = np.zeros_like(P)
        dP[:, k] = h * np.maximum(1.0, np.abs(P[:, k]))
        dU = primitive_to_conservative(P + dP, gamma) - primitive_to_conservative(P - dP, gamma)
        fd[:, k] = (dU * lam).sum(axis=1) / (2.0 * dP[:, k])
    np.testing.assert_allclose(got, fd, rtol=1e-7, atol=1e-8)
