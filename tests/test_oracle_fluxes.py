"""The oracle's face fluxes as functions (no GPU): the reference's
consistency test (tests/test_solver.py:145-155, F(u, u) = f(u) . n for equal
states) for Rusanov, HLLC in both branch orders and Roe, plus the fluxes'
symmetry under exchanging the two sides and reversing the normal."""

import numpy as np
import pytest

from oracle.oracle import FACE_FLUXES, face_fluxes


def _physical_flux(q, n, gamma):
    """euler.physical_flux (euler.py:43-57): the normal flux of primitive
    states q across normals n."""
    r, u, v, p = q.T
    un = u * n[:, 0] + v * n[:, 1]
    E = p / (gamma - 1.0) + 0.5 * r * (u * u + v * v)
    return np.column_stack((r * un, r * u * un + p * n[:, 0], r * v * un + p * n[:, 1], (E + p) * un))


@pytest.mark.parametrize("kind", sorted(FACE_FLUXES))
def test_numerical_fluxes_return_the_physical_flux_for_equal_states(kind):
    states = np.array(((1.2, 0.4, -0.3, 1.1), (0.9, -0.2, 0.5, 0.8), (1.0, 0.0, 0.0, 1.0)))
    normals = np.array(((1.0, 0.0), (0.0, 1.0), (0.6, 0.8)))
    flux = face_fluxes(kind, states, states, normals, 1.4)
    np.testing.assert_allclose(flux, _physical_flux(states, normals, 1.4), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("kind", sorted(FACE_FLUXES))
def test_fluxes_are_antisymmetric_under_side_exchange(kind):
    """F(L, R, n) = -F(R, L, -n): the face flux seen from the other cell."""
    rng = np.random.default_rng(5)
    n = 200
    L = np.column_stack((rng.uniform(0.5, 2.0, n), rng.uniform(-1.5, 1.5, n), rng.uniform(-1.5, 1.5, n),
                         rng.uniform(0.5, 2.0, n)))
    R = np.column_stack((rng.uniform(0.5, 2.0, n), rng.uniform(-1.5, 1.5, n), rng.uniform(-1.5, 1.5, n),
                         rng.uniform(0.5, 2.0, n)))
    theta = rng.uniform(0.0, 2.0 * np.pi, n)
    normals = np.column_stack((np.cos(theta), np.sin(theta)))
    forward = face_fluxes(kind, L, R, normals, 1.4)
    backward = face_fluxes(kind, R, L, -normals, 1.4)
    np.testing.assert_allclose(forward, -backward, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("kind", ("Rusanov", "HLLC", "Roe"))
def test_fluxes_equal_the_references_bit_for_bit(kind):
    """tests/golden/fluxes.npz: the reference's euler.numerical_flux on 1,000
    random faces (subsonic and supersonic, both directions)."""
    from conftest import ROOT

    data = np.load(ROOT / "tests" / "golden" / "fluxes.npz")
    np.testing.assert_array_equal(face_fluxes(kind, data["L"], data["R"], data["normals"], 1.4), data[kind])
