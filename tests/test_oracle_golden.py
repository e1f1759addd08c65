"""The oracle against the reference's own outputs (golden fixtures): pins the
oracle before it is used to check the GPU path."""

import numpy as np
import pytest

from conftest import load_fixture, residual_keys, settings_for, solve_settings
from oracle.oracle import Oracle

RESIDUAL_FIXTURES = ("residual_riemann16.npz", "residual_periodic_mixed.npz", "residual_channel.npz")
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
