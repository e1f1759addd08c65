"""MUSCL-parabolic reconstruction of the oracle against the reference's own
outputs (golden fixtures) and against the quadratic-exactness property the
reference tests (test_solver.py:843-872).

The reference solves each cell's 5x5 normal equations with LAPACK (through
np.linalg.solve) and gates them with an SVD rank; the oracle restates the
solve as Gaussian elimination with partial pivoting, so its values agree to
rounding (a few 1e-15 relative), not bit for bit.  Rank decisions agree: the
rank-deficient strip falls back to linear reconstruction in every cell, bit
for bit.
"""

import numpy as np
import pytest

from conftest import load_fixture, residual_keys, settings_for, solve_settings
from oracle.oracle import Oracle

FIXTURES = ("parabolic_riemann16.npz", "parabolic_periodic_mixed.npz", "parabolic_channel.npz",
            "parabolic_strip.npz")
LIMITERS = ("Barth-Jespersen", "Minmod", "Van Leer", "Venkatakrishnan")
TOL = 1e-13  # relative to the largest magnitude of each compared array


def _close(a, b, tol=TOL):
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_parabolic_reconstruction_matches_reference(name):
    data, geom = load_fixture(name)
    orc = Oracle(geom)
    P = orc.primitive(data["U"], 1.4)
    for code, limiter in enumerate(LIMITERS):
        g, k, f = orc.parabolic_reconstruction(P, limiter)
        assert _close(g, data[f"pgrad|{code}"]), limiter
        assert _close(k, data[f"pcurv|{code}"]), limiter
        assert _close(f, data[f"pfactors|{code}"]), limiter
        # the same cells fall back to linear reconstruction (zero curvature)
        np.testing.assert_array_equal(np.all(k == 0, axis=(1, 2)),
                                      np.all(data[f"pcurv|{code}"] == 0, axis=(1, 2)))


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_parabolic_residual_matches_reference(name):
    data, geom = load_fixture(name)
    orc = Oracle(geom)
    keys = residual_keys(data)
    assert len(keys) == 24
    for key in keys:
        R = orc.residual(data["U"], settings_for(key))
        assert _close(R, data[key]), key
        if name == "parabolic_strip.npz":  # every cell takes the linear path
            np.testing.assert_array_equal(R, data[key], err_msg=key)


def test_oracle_parabolic_solve_matches_reference():
    data, geom = load_fixture("solve_vortex12_rk3_parabolic.npz")
    s = solve_settings(data)
    orc = Oracle(geom)
    U, t = orc.solve(orc.conservative(data["P0"], s.gamma), s, int(data["steps"]))
    assert _close(orc.primitive(U, s.gamma), data["P_final"], 1e-12)
    assert abs(t - float(data["time"])) <= 1e-14 * float(data["time"])


def test_parabolic_reconstruction_recovers_quadratic_field():
    """test_solver.py:843-872, with the geometry built for MUSCL parabolic
    (the stencil exists only then, test_solver.py:1608-1629)."""
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import periodic_case

    case = periodic_case(6, 6)
    case.numerics.reconstruction = "MUSCL parabolic"
    g = build_geometry(case.mesh, case)
    x, y = np.asarray(g.centers).T
    P = np.column_stack((10.0 + x * x + 2.0 * x * y + 3.0 * y * y, np.full_like(x, 0.2), np.full_like(x, -0.1),
                         np.ones_like(x)))
    grad, curv, fac = Oracle(g).parabolic_reconstruction(P, "Barth-Jespersen")
    c = 3 * 6 + 3
    np.testing.assert_allclose(grad[c, 0], (2.0 * x[c] + 2.0 * y[c], 2.0 * x[c] + 6.0 * y[c]), rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(curv[c, 0], (2.0, 2.0, 6.0), rtol=1e-10, atol=1e-10)
    assert fac[c, 0] == pytest.approx(1.0)


@pytest.mark.parametrize("mesh", ("vortex_half", "bump", "periodic_permuted", "box_all"))
def test_compiled_two_ring_stencil_equals_the_restated_search(mesh):
    """The library's threaded two-ring search (mcfd_host_parabolic_stencil)
    returns the entries of the Python restatement of _parabolic_stencil
    (solver.py:2241-2291) in the same order, on periodic meshes (offsets
    across the period, where the rounded-offset keys separate images of one
    cell), a stretched wall-bounded mesh, randomly numbered cells and an
    all-triangle box."""
    from meshcfd_gb300 import _lib
    from meshcfd_gb300.geometry import build_geometry, parabolic_stencil
    from meshcfd_gb300.meshes import box_mesh, bump_case, periodic_case, permute_mesh, vortex_case
    from meshcfd_gb300.model import Case

    if mesh == "vortex_half":
        case, _ = vortex_case(24, split="half")
    elif mesh == "bump":
        case, _ = bump_case(24, 12)
    elif mesh == "periodic_permuted":
        case = periodic_case(20, 20, split="half", jitter=0.2, seed=5)
        rng = np.random.default_rng(3)
        case.mesh = permute_mesh(case.mesh, rng.permutation(len(case.mesh.cells)),
                                 rng.permutation(len(case.mesh.faces)))
    else:
        case = Case(name="box", mesh=box_mesh(14, 9, 2.0, 1.0, split="all", jitter=0.2, seed=2))
    g = build_geometry(case.mesh, case)
    points = np.asarray(case.mesh.points, dtype=float)
    scale = max(float(np.ptp(points[:, 0])), float(np.ptp(points[:, 1])), 1e-12)
    args = (len(g.areas), np.asarray(g.gradient_sources), np.asarray(g.gradient_neighbours),
            np.asarray(g.gradient_dx), np.asarray(g.gradient_dy), scale)
    ref = parabolic_stencil(*args)
    got = _lib.native().parabolic_stencil(*args)
    assert len(ref[0]) > 6 * len(g.areas)
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)
