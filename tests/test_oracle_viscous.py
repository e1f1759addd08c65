"""Laminar viscous terms of the oracle against the reference's own outputs
(golden fixtures): viscous gradients and residual, full residuals with the
viscous terms, stable time steps with the diffusion term, and a short RK3
solve; plus the geometry builder's viscous fields."""

import numpy as np
import pytest

from conftest import load_fixture, residual_keys, solve_settings, viscous_settings_for
from oracle.oracle import Oracle

KINDS = ("noslip", "mixed", "periodic")


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("kind", KINDS)
def test_oracle_viscous_terms_match_reference(kind):
    from oracle.viscous import viscous_gradients, viscous_residual

    data, geom = load_fixture(f"viscous_{kind}.npz")
    orc = Oracle(geom)
    P = orc.primitive(data["U"], 1.4)
    keys = residual_keys(data)
    assert keys
    models = sorted({k.split("|")[5] for k in keys})
    for key in keys:
        s = viscous_settings_for(key, data)
        assert _rel(orc.residual(data["U"], s), data[key]) <= 1e-14, key
    for model in models:
        s = viscous_settings_for(next(k for k in keys if k.endswith(model)), data)
        assert _rel(viscous_gradients(P, geom, s, orc), data[f"G|{model}"]) <= 1e-14
        assert _rel(viscous_residual(P, geom, s, orc, orc.divergence), data[f"V|{model}"]) <= 1e-13
        s.cfl = 0.7
        assert _rel(orc.stable_time_steps(P, s), data[f"dt|{model}"]) <= 1e-15


def test_oracle_viscous_solve_matches_reference():
    data, geom = load_fixture("solve_viscous_noslip_rk3.npz")
    s = solve_settings(data)
    orc = Oracle(geom)
    U, t = orc.solve(orc.conservative(data["P0"], s.gamma), s, int(data["steps"]))
    assert _rel(orc.primitive(U, s.gamma), data["P_final"]) <= 1e-13
    assert abs(t - float(data["time"])) <= 1e-15 * float(data["time"])


@pytest.mark.parametrize("kind", KINDS)
def test_geometry_builder_viscous_fields_match_reference(kind):
    from make_golden import viscous_case
    from meshcfd_gb300.geometry import build_geometry

    data, ref = load_fixture(f"viscous_{kind}.npz")
    case = viscous_case(kind)
    case.numerics.reconstruction = "MUSCL parabolic"
    g = build_geometry(case.mesh, case)
    np.testing.assert_array_equal(g.diffusive_boundary_faces, ref.diffusive_boundary_faces)
    np.testing.assert_array_equal(np.asarray(g.patch_ids), ref.patch_ids)
    assert {k: v for k, v in g.patch_kinds.items()} == ref.patch_kinds
    assert len(g.wall_thermal_boundaries) == len(ref.wall_thermal_boundaries)
    for a, b in zip(g.wall_thermal_boundaries, ref.wall_thermal_boundaries):
        np.testing.assert_array_equal(np.asarray(a.faces), b.faces)
        assert (a.condition, a.value, a.patch_name, a.mechanical_condition) == \
            (b.condition, b.value, b.patch_name, b.mechanical_condition)
