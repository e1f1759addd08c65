"""The oracle against the reference's own outputs (golden fixtures): pins the
oracle before it is used to check the GPU path."""

import numpy as np
import pytest

from conftest import load_fixture, residual_keys, settings_for, solve_settings
from oracle.oracle import Oracle

RESIDUAL_FIXTURES = ("residual_riemann16.npz", "residual_periodic_mixed.npz", "residual_channel.npz",
                     "residual_bump.npz", "residual_ogrid.npz")
SOLVE_FIXTURES = ("solve_riemann16_euler.npz", "solve_vortex12_rk3.npz", "solve_channel_rk4_local.npz",
                  "solve_channel_rk2_vanleer.npz")


@pytest.mark.parametrize("name", RESIDUAL_FIXTURES)
def test_oracle_residual_matches_reference(name):
    data, geom = load_fixture(name)
    orc = Oracle(geom)
    far = len(geom.far_field_faces) > 0
    for key in residual_keys(data):
        R = orc.residual(data["U"], settings_for(key))
        ref = data[key]
        if far:
            # pow() of the far-field state: libm vs the reference's NumPy SIMD
            # power differ in the last place on a few faces.
            assert np.abs(R - ref).max() <= 1e-15 * np.abs(ref).max(), key
        else:
            np.testing.assert_array_equal(R, ref, err_msg=key)


@pytest.mark.parametrize("name", RESIDUAL_FIXTURES)
def test_oracle_time_steps_and_limiter_match_reference(name):
    data, geom = load_fixture(name)
    orc = Oracle(geom)
    from meshcfd_gb300.model import NumericalSettings

    P = orc.primitive(data["U"], 1.4)
    dt = orc.stable_time_steps(P, NumericalSettings(cfl=float(data["cfl"])))
    if len(geom.far_field_faces):
        np.testing.assert_allclose(dt, data["dt_cells"], rtol=1e-15, atol=0)
    else:
        np.testing.assert_array_equal(dt, data["dt_cells"])
    for code, limiter in enumerate(("Barth-Jespersen", "Minmod", "Van Leer", "Venkatakrishnan")):
        g, f = orc.gradients_and_factors(P, limiter)
        np.testing.assert_array_equal(g, data[f"grad|{code}"])
        np.testing.assert_array_equal(f, data[f"factors|{code}"])


@pytest.mark.parametrize("name", SOLVE_FIXTURES)
def test_oracle_solve_matches_reference(name):
    data, geom = load_fixture(name)
    orc = Oracle(geom)
    s = solve_settings(data)
    U0 = orc.conservative(data["P0"], s.gamma)
    U, time = orc.solve(U0, s, int(data["steps"]))
    P = orc.primitive(U, s.gamma)
    ref = data["P_final"]
    assert np.abs(P - ref).max() <= 1e-13 * np.abs(ref).max()
    if "riemann" not in name:
        np.testing.assert_array_equal(P, ref)
        assert time == float(data["time"])
    else:
        assert abs(time - float(data["time"])) <= 1e-14 * float(data["time"])


@pytest.mark.parametrize("name", ("implicit_channel.npz", "implicit_periodic.npz"))
def test_oracle_implicit_matches_reference(name):
    """The oracle's restatement of the implicit Euler pieces against the
    reference: LU-SGS application, the finite-difference operator, and the
    implicit solve_case."""
    from dataclasses import replace

    from conftest import solve_settings
    from oracle.implicit import ImplicitOracle

    data, geom = load_fixture(name)
    s = solve_settings(data)
    imp = ImplicitOracle(geom)
    first = replace(s, reconstruction="First order")
    M = imp.preconditioner(data["P0"], first, data["dt_cells"])
    np.testing.assert_allclose(M.matvec(data["v"]), data["lusgs_v"], rtol=1e-13, atol=1e-13 * np.abs(data["lusgs_v"]).max())
    U = data["U"]
    rate = imp.orc.residual(U, first)
    op = imp.operator(U, rate, data["scales"][None, :], data["dt_cells"], first)
    np.testing.assert_allclose(op.matvec(data["v"]), data["operator_v"], rtol=1e-12,
                               atol=1e-12 * np.abs(data["operator_v"]).max())
    # the implicit loop (local steady or global adaptive time step)
    Uc = U.copy()
    time = 0.0
    for _ in range(int(data["steps"])):
        P = imp.orc.primitive(Uc, s.gamma)
        dt = imp.orc.stable_time_steps(P, s)
        step = dt if s.time_step_mode == "Local (steady)" else float(np.min(dt))
        Uc, used = imp.step(Uc, step, s)
        time += float(np.mean(used))
    P = imp.orc.primitive(Uc, s.gamma)
    assert np.abs(P - data["P_final"]).max() <= 1e-10 * np.abs(data["P_final"]).max()
    assert abs(time - float(data["time"])) <= 1e-12 * float(data["time"])


def test_oracle_implicit_step_on_the_bump_recipe_matches_reference():
    """tests/golden/implicit_bump.npz: the reference's implicit-Euler step on
    a 16x8 bump channel (Roe, MUSCL linear, Barth-Jespersen, local CFL 200,
    GMRES(30) to 1e-3, LU-SGS) halves its time step 9 times before its
    Newton solve converges; the oracle takes the same steps to the same
    state."""
    from conftest import ROOT
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import bump_case
    from oracle.implicit import ImplicitOracle

    data = np.load(ROOT / "tests" / "golden" / "implicit_bump.npz")
    case, _ = bump_case(16, 8)
    g = build_geometry(case.mesh, case)
    out, used = ImplicitOracle(g).step(data["U"], data["dt"], case.numerics)
    np.testing.assert_array_equal(used, data["used"])
    np.testing.assert_array_equal(used, data["dt"] * 0.5**9)
    assert np.abs(out - data["U_next"]).max() <= 1e-12 * np.abs(data["U_next"]).max()
