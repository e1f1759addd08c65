"""Pressure-inlet and mass-flow boundaries of the oracle against the
reference's own outputs (golden fixtures), and the boundary-state checks.

The reference evaluates Python-float powers with libm and NumPy array powers
with NumPy's own SIMD code; the oracle uses libm for both, so values agree to
the last place (about 1e-15 relative), not bit for bit.
"""

import numpy as np
import pytest

from conftest import load_fixture, residual_keys, settings_for, solve_settings
from oracle.oracle import Oracle, OracleError

FIXTURES = ("bc_pinlet.npz", "bc_massflow.npz")


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_boundary_residuals_and_time_steps_match_reference(name):
    from meshcfd_gb300.model import NumericalSettings

    data, geom = load_fixture(name)
    orc = Oracle(geom)
    keys = residual_keys(data)
    assert len(keys) == 12
    for key in keys:
        assert _rel(orc.residual(data["U"], settings_for(key)), data[key]) <= 1e-14, key
    dt = orc.stable_time_steps(orc.primitive(data["U"], 1.4), NumericalSettings(cfl=float(data["cfl"])))
    assert _rel(dt, data["dt_cells"]) <= 1e-14


@pytest.mark.parametrize("name", ("solve_pinlet_rk3.npz", "solve_massflow_rk3.npz"))
def test_oracle_boundary_solve_matches_reference(name):
    data, geom = load_fixture(name)
    s = solve_settings(data)
    orc = Oracle(geom)
    U, t = orc.solve(orc.conservative(data["P0"], s.gamma), s, int(data["steps"]))
    assert _rel(orc.primitive(U, s.gamma), data["P_final"]) <= 1e-13
    assert abs(t - float(data["time"])) <= 1e-15 * float(data["time"])


def _one_cell(kinds):
    """One-cell box (test_solver.py:134-143 without periodic pairs) with the
    given boundary kinds per patch index (0 bottom, 1 right, 2 top, 3 left)."""
    from meshcfd_gb300.meshes import periodic_case

    case = periodic_case(1, 1)
    case.periodic_pairs.clear()
    case.numerics.gas_constant = 1.0
    for c in case.boundary_conditions:
        c.kind = "Wall"
        c.mechanical_condition = "Slip"
    for k, (kind, values) in kinds.items():
        case.boundary_conditions[k].kind = kind
        case.boundary_conditions[k].values = values
    return case


def test_pressure_inlet_reconstructs_matching_subsonic_flow():
    """test_solver.py:953-988."""
    from meshcfd_gb300.geometry import build_geometry

    tt = 1.0 + 0.2 ** 2 / (2.0 * 3.5)
    pt = tt ** (1.4 / 0.4)
    case = _one_cell({3: ("Pressure Inlet", {"pressure": pt, "temperature": tt, "velocity_x": 1.0,
                                            "velocity_y": 0.0})})
    orc = Oracle(build_geometry(case.mesh, case))
    interior = np.array(((1.0, 0.2, 0.0, 1.0),))
    np.testing.assert_allclose(orc.boundary_states(0, interior, 1.4, 1.0), interior, rtol=1e-12, atol=1e-12)
    with pytest.raises(OracleError, match="supersonic inflow"):
        orc.boundary_states(0, np.array(((1.0, 2.0, 0.0, 1.0),)), 1.4, 1.0)


def test_mass_flow_inlet_satisfies_integrated_flow_rate():
    """test_solver.py:991-1025."""
    from meshcfd_gb300.geometry import build_geometry

    case = _one_cell({3: ("Mass Flow Inlet", {"mass_flow": 0.25, "temperature": 2.0, "velocity_x": 1.0,
                                             "velocity_y": 0.0})})
    g = build_geometry(case.mesh, case)
    b = g.mass_flow_inlets[0]
    normals = np.asarray(g.face_normals)[b.faces]
    lengths = np.asarray(g.face_lengths)[b.faces]
    states = Oracle(g).boundary_states(0, np.array(((1.0, 0.0, 0.0, 1.0),)), 1.4, 1.0)
    flow = np.sum(states[:, 0] * -(states[:, 1:3] * normals).sum(axis=1) * lengths)
    assert flow == pytest.approx(0.25, rel=1e-12)
    np.testing.assert_allclose(states[:, 3], 1.0)


def test_mass_flow_outlet_preserves_pressure_density_and_tangential_velocity():
    """test_solver.py:1028-1046."""
    from meshcfd_gb300.geometry import build_geometry

    case = _one_cell({1: ("Mass Flow Outlet", {"mass_flow": 0.6})})
    g = build_geometry(case.mesh, case)
    b = g.mass_flow_outlets[0]
    normals = np.asarray(g.face_normals)[b.faces]
    lengths = np.asarray(g.face_lengths)[b.faces]
    interior = np.array(((2.0, 0.4, 0.3, 1.2),))
    states = Oracle(g).boundary_states(0, interior, 1.4, 1.0)
    assert np.sum(states[:, 0] * (states[:, 1:3] * normals).sum(axis=1) * lengths) == pytest.approx(0.6)
    np.testing.assert_allclose(states[:, (0, 3)], interior[:, (0, 3)])
    np.testing.assert_allclose(states[:, 2], interior[:, 2])


@pytest.mark.parametrize("kind", ("Pressure Inlet", "Mass Flow Inlet"))
def test_inlets_reject_direction_pointing_out_of_domain(kind):
    """test_solver.py:1063-1079."""
    from meshcfd_gb300.geometry import build_geometry

    values = ({"pressure": 101325.0, "temperature": 288.15} if kind == "Pressure Inlet"
              else {"mass_flow": 0.2, "temperature": 288.15})
    values.update({"velocity_x": -1.0, "velocity_y": 0.0})
    case = _one_cell({3: (kind, values)})
    orc = Oracle(build_geometry(case.mesh, case))
    with pytest.raises(OracleError, match="direction must point into the domain"):
        orc.boundary_states(0, np.array(((1.0, 0.0, 0.0, 1.0),)), 1.4, 1.0)


def test_far_field_characteristics_select_incoming_and_outgoing_information():
    """test_solver.py:1149-1166 on the oracle: supersonic outflow keeps the
    interior state, supersonic inflow takes the far-field state, subsonic
    outflow takes the normal velocity from the two Riemann invariants and the
    tangential velocity and entropy from the interior."""
    from oracle.oracle import far_field_states

    interior = np.array(((1.0, 3.0, 0.0, 1.0), (1.0, 0.2, 0.0, 1.0), (1.0, -3.0, 0.0, 1.0)))
    far = np.array(((2.0, 0.0, 0.0, 2.0), (2.0, 0.4, 0.0, 2.0), (2.0, 0.0, 0.0, 2.0)))
    normals = np.array(((1.0, 0.0), (1.0, 0.0), (1.0, 0.0)))
    ext = far_field_states(interior, far, normals, 1.4)
    np.testing.assert_array_equal(ext[0], interior[0])
    np.testing.assert_array_equal(ext[2], far[2])
    assert ext[1, 1] == pytest.approx(0.3)
    assert ext[1, 2] == pytest.approx(interior[1, 2])
    assert ext[1, 3] / ext[1, 0] ** 1.4 == pytest.approx(interior[1, 3] / interior[1, 0] ** 1.4)
