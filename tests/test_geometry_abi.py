"""Host side: geometry builder vs the reference's geometry (golden), mesh
generators, and the C ABI library's exports (no GPU needed)."""

import re
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT, fixture_mesh, load_fixture

FIELDS = ("centers", "areas", "face_centers", "face_normals", "face_lengths", "interior_faces",
          "interior_owner_offsets", "interior_neighbour_offsets", "wall_faces", "periodic_faces_a",
          "periodic_faces_b", "velocity_inlet_faces", "velocity_inlet_states", "pressure_outlet_faces",
          "pressure_outlet_pressures", "far_field_faces", "far_field_states", "gradient_sources",
          "gradient_neighbours", "gradient_coefficients_x", "gradient_coefficients_y", "limiter_cells",
          "limiter_dx", "limiter_dy")


def _case_for(name):
    from make_golden import channel_case
    from meshcfd_gb300.meshes import periodic_case, riemann_case

    return {"riemann16": lambda: riemann_case(16)[0],
            "periodic_mixed": lambda: periodic_case(8, 6, split="half", jitter=0.25, seed=2),
            "channel": channel_case}[name]()


@pytest.mark.parametrize("name", ("riemann16", "periodic_mixed", "channel"))
def test_geometry_builder_is_bit_exact(name):
    from meshcfd_gb300.geometry import build_geometry

    data, ref = load_fixture(f"residual_{name}.npz")
    case = _case_for(name)
    # the generator reproduces the fixture's mesh exactly
    mesh = fixture_mesh(data)
    np.testing.assert_array_equal(np.asarray(case.mesh.points), mesh.points)
    np.testing.assert_array_equal(np.asarray(case.mesh.faces), mesh.faces)
    g = build_geometry(case.mesh, case)
    for field in FIELDS:
        np.testing.assert_array_equal(np.asarray(getattr(g, field)).reshape(np.shape(getattr(ref, field))),
                                      getattr(ref, field), err_msg=field)


@pytest.mark.parametrize("name", ("riemann16", "periodic_mixed", "channel"))
def test_oracle_geometry_loops_are_bit_exact(name):
    """The oracle's restatement of the cell / face loops (what the CPU
    reference arm builds its geometry with, without the product library)
    against the reference's own arrays, and refusing degenerate elements with
    the reference's messages."""
    from meshcfd_gb300.geometry import build_geometry
    from oracle.oracle import GeometryHost, OracleError

    data, ref = load_fixture(f"residual_{name}.npz")
    case = _case_for(name)
    g = build_geometry(case.mesh, case, host=GeometryHost())
    for field in FIELDS:
        np.testing.assert_array_equal(np.asarray(getattr(g, field)).reshape(np.shape(getattr(ref, field))),
                                      getattr(ref, field), err_msg=field)
    points = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0]])
    with pytest.raises(OracleError, match="Cell 0 has zero or invalid area"):
        GeometryHost.cell_geometry(np.array([0, 3]), np.array([0, 1, 2]), points)
    with pytest.raises(OracleError, match="Face 0 has zero or invalid length"):
        GeometryHost.face_geometry(np.array([[0, 0]]), points, np.zeros((1, 2)), np.array([0]))


def test_workload_mesh_sizes():
    from meshcfd_gb300.meshes import riemann_case, vortex_case

    case, P = riemann_case(128)
    m = case.mesh
    assert len(m.cells) == 32768 and len(m.faces) == 49408
    assert int((np.asarray(m.face_neighbours) >= 0).sum()) == 48896
    assert P.shape == (32768, 4)
    v, _ = vortex_case(32)
    assert len(v.mesh.cells) == 32 * 32 + 32 * 32 // 2


def test_bump_channel_mesh():
    """The bump-channel configuration at full size: 512 x 256 quads, the arc's
    crest at 10 % of the chord, wall / far-field / outlet face counts, every
    cell of positive area (the rows stretched by 1.05 toward the wall)."""
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import bump_case

    case, P = bump_case()
    g = build_geometry(case.mesh, case)
    assert len(g.areas) == 131072 and P.shape == (131072, 4)
    assert (len(g.wall_faces), len(g.far_field_faces), len(g.pressure_outlet_faces)) == (512, 768, 256)
    assert float(np.min(g.areas)) > 0.0
    points = np.asarray(case.mesh.points)
    assert abs(points[:513, 1].max() - 0.1) < 1e-5  # the wall row; x = 0.5 is a grid line
    assert case.numerics.flux == "Roe" and case.numerics.limiter == "Barth-Jespersen"


def test_ogrid_mesh():
    """The adjoint configuration's O-grid at full size: 1024 x 512 quads
    between the cylinder (radius 0.5) and the square [-10, 10]^2, 1,024 wall
    and 1,024 far-field faces, every cell of positive area."""
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import ogrid_case

    case, P = ogrid_case(1024, 512)
    g = build_geometry(case.mesh, case)
    assert len(g.areas) == 524288 and P.shape == (524288, 4)
    assert (len(g.wall_faces), len(g.far_field_faces)) == (1024, 1024)
    assert float(np.min(g.areas)) > 0.0
    points = np.asarray(case.mesh.points)
    np.testing.assert_allclose(np.linalg.norm(points[:1024], axis=1), 0.5, rtol=1e-15)
    np.testing.assert_array_equal(np.abs(points[-1024:]).max(axis=1), 10.0)


def test_periodic_matching_rejects_mismatch():
    from meshcfd_gb300.errors import SolverError
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import periodic_case

    case = periodic_case(4, 3)
    case.periodic_pairs[0] = type(case.periodic_pairs[0])(1, 3, "x", 2.0)  # stale pitch
    with pytest.raises(SolverError, match="stale axis or pitch"):
        build_geometry(case.mesh, case)


def _declared_symbols():
    text = (ROOT / "include" / "meshcfd_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mcfd_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from meshcfd_gb300 import _lib

    native = _lib.native()
    declared = _declared_symbols()
    assert len(declared) >= 10
    for name in declared:
        assert hasattr(native.lib, name), name
    assert set(declared) == set(_lib.SIGNATURES), "ctypes signatures out of sync with the header"
    assert native.mcfd_abi_version() == _lib.ABI_VERSION == 6
    assert native.mcfd_error_string(3) == b"option not supported by the GPU path"


def test_host_geometry_helpers_reject_degenerate_cells():
    from meshcfd_gb300 import _lib
    from meshcfd_gb300.errors import SolverError

    native = _lib.native()
    points = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0]])
    with pytest.raises(SolverError, match="Cell 0 has zero or invalid area"):
        native.cell_geometry(np.array([0, 3]), np.array([0, 1, 2]), points)
    with pytest.raises(SolverError, match="Face 0 has zero or invalid length"):
        native.face_geometry(np.array([[0, 0]]), points, np.zeros((1, 2)), np.array([0]))


MALFORMED = {
    # name: (mutation of the descriptor's arrays / fields, expected return code)
    "no cells": (lambda d, k: setattr(d, "n_cells", 0), 1),
    "cells beyond the 2^30 index limit": (lambda d, k: setattr(d, "n_cells", (1 << 30) + 1), 1),
    "faces beyond the 2^30 index limit": (lambda d, k: setattr(d, "n_faces", (1 << 30) + 1), 1),
    "null areas": (lambda d, k: setattr(d, "areas", None), 1),
    "owner out of range": (lambda d, k: k["owners"].__setitem__(0, d.n_cells), 4),
    "neighbour out of range": (lambda d, k: k["neighbours"].__setitem__(k["interior_faces"][0], d.n_cells), 4),
    "interior faces unsorted": (lambda d, k: k["interior_faces"].__setitem__(slice(0, 2), k["interior_faces"][1::-1]), 4),
    "far-field face with a neighbour": (lambda d, k: k["far_field_faces"].__setitem__(0, k["interior_faces"][0]), 4),
    "gradient neighbour negative": (lambda d, k: k["gradient_neighbours"].__setitem__(0, -1), 4),
    "limiter cell out of range": (lambda d, k: k["limiter_cells"].__setitem__(0, d.n_cells), 4),
    "limiter count": (lambda d, k: setattr(d, "n_limiter", d.n_limiter - 1), 4),
    "zero area": (lambda d, k: k["areas"].__setitem__(3, 0.0), 4),
}


@pytest.mark.parametrize("name", sorted(MALFORMED))
def test_geometry_create_rejects_malformed_descriptors(name):
    """mcfd_geom_create validates every index before it touches the device,
    so no kernel can read out of bounds; malformed descriptors return
    MCFD_E_ARG (1) or MCFD_E_GEOMETRY (4) without a GPU."""
    import ctypes as C

    from meshcfd_gb300 import _lib
    from meshcfd_gb300.device import geometry_descriptor
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import riemann_case

    case, _ = riemann_case(6)
    desc, keep, _ = geometry_descriptor(build_geometry(case.mesh, case))
    assert desc.n_far_field > 0 and desc.n_interior > 1
    mutate, expected = MALFORMED[name]
    mutate(desc, keep)
    handle = C.c_void_p()
    assert _lib.native().mcfd_geom_create(C.byref(desc), C.byref(handle)) == expected
    assert handle.value is None


def test_config_mapping_rejects_unsupported_models():
    from meshcfd_gb300.device import make_config
    from meshcfd_gb300.model import NumericalSettings

    assert make_config(NumericalSettings(viscosity_model="Sutherland")).viscosity_model == 2
    with pytest.raises(NotImplementedError):
        make_config(NumericalSettings(turbulence_model="SST"))
    assert make_config(NumericalSettings(reconstruction="MUSCL parabolic")).reconstruction == 2
    cfg = make_config(NumericalSettings(flux="Roe", limiter="Van Leer", reconstruction="MUSCL linear"))
    assert (cfg.flux, cfg.limiter, cfg.reconstruction) == (2, 2, 1)


@pytest.mark.parametrize("name", ("riemann16", "periodic_mixed", "channel"))
def test_parabolic_stencil_is_bit_exact(name):
    """The two-ring stencil (solver.py:2241-2291) of a geometry built for
    MUSCL parabolic, against the reference's own."""
    from meshcfd_gb300.geometry import build_geometry

    data, ref = load_fixture(f"parabolic_{name}.npz")
    case = _case_for(name)
    case.numerics.reconstruction = "MUSCL parabolic"
    g = build_geometry(case.mesh, case)
    for field in ("parabolic_sources", "parabolic_neighbours", "parabolic_dx", "parabolic_dy"):
        np.testing.assert_array_equal(np.asarray(getattr(g, field)), getattr(ref, field), err_msg=field)
