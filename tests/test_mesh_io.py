"""The MeshCAD JSON mesh reader against the reference's own reader
(tests/golden/meshio.json, made by make_golden.py from io/mesh_io.py): the
same cell loops and serialisation on valid inputs, the same message for
every rejected input; the reference's own reader tests
(tests/test_mesh_io.py) restated; the geometry of a mesh read back from its
JSON equal to the original's, bit for bit."""

import copy
import json
from pathlib import Path

import numpy as np
import pytest

from make_golden import MESH_MUTATIONS, MESHIO_BASES, meshio_square
from meshcfd_gb300 import mesh_io
from meshcfd_gb300.mesh_io import MeshImportError, load_mesh, mesh_from_dict, mesh_to_dict

GOLDEN = json.loads((Path(__file__).parent / "golden" / "meshio.json").read_text())


def _cells(mesh):
    return [list(mesh.cells[c]) for c in range(len(mesh.cells))]


@pytest.mark.parametrize("name", sorted(GOLDEN["valid"]))
def test_reader_matches_reference_on_valid_meshes(name):
    entry = GOLDEN["valid"][name]
    mesh = mesh_from_dict(copy.deepcopy(entry["data"]))
    assert _cells(mesh) == entry["cells"]
    assert mesh_to_dict(mesh) == entry["to_dict"]
    # and the serialisation reads back to the same mesh
    again = mesh_from_dict(mesh_to_dict(mesh))
    assert _cells(again) == entry["cells"]
    assert mesh_to_dict(again) == entry["to_dict"]


@pytest.mark.parametrize("name,base,mutate", MESH_MUTATIONS, ids=[m[0] for m in MESH_MUTATIONS])
def test_reader_rejects_as_the_reference_does(name, base, mutate):
    data = MESHIO_BASES[base]()
    mutate(data)
    with pytest.raises(MeshImportError) as error:
        mesh_from_dict(data)
    assert str(error.value) == GOLDEN["errors"][name]


# ---- the reference's reader tests (tests/test_mesh_io.py:31-86), restated

def test_meshcad_mesh_import_and_export_round_trip():
    data = meshio_square()
    mesh = mesh_from_dict(copy.deepcopy(data))
    assert tuple(mesh.points[2]) == (1.0, 1.0)
    assert _cells(mesh) == [[0, 1, 2, 3]]
    assert [patch.name for patch in mesh.patches] == ["bottom", "right", "top", "left"]
    assert mesh_to_dict(mesh) == data


def test_mesh_import_rejects_open_cell():
    data = meshio_square()
    data["cells"]["face_signs"][0][-1] = -1
    with pytest.raises(MeshImportError, match="closed node loop"):
        mesh_from_dict(data)


def test_mesh_import_rejects_non_finite_coordinates():
    data = meshio_square()
    data["nodes"]["coordinates"][0][0] = float("nan")
    with pytest.raises(MeshImportError, match="finite"):
        mesh_from_dict(data)


def test_mesh_boundary_curve_metadata_round_trips_and_validates():
    data = meshio_square()
    data["boundary_curves"] = [
        {"geometry": {"type": "arc", "center": [0.5, 0.5], "radius": 2 ** 0.5 / 2,
                      "start_angle": -3 * 3.141592653589793 / 4, "end_angle": -3.141592653589793 / 4},
         "parameters": [0.0, 1.0], "patch_id": 0},
        None, None, None,
    ]
    mesh = mesh_from_dict(data)
    assert mesh.face_curves[0] is not None
    assert mesh.face_curves[0].geometry["type"] == "arc"
    assert mesh_to_dict(mesh)["boundary_curves"] == data["boundary_curves"]
    assert mesh_to_dict(mesh_from_dict(mesh_to_dict(mesh))) == mesh_to_dict(mesh)
    data["boundary_curves"][0]["parameters"] = [0.0, 0.5]
    with pytest.raises(MeshImportError, match="does not match its face nodes"):
        mesh_from_dict(data)


# ---- files and the path the reader feeds

def test_load_mesh_reads_files_and_reports_bad_ones(tmp_path):
    good = tmp_path / "square.json"
    good.write_text(json.dumps(meshio_square()))
    assert _cells(load_mesh(good)) == [[0, 1, 2, 3]]
    with pytest.raises(MeshImportError, match="Could not read mesh file"):
        load_mesh(tmp_path / "missing.json")
    bad = tmp_path / "bad.json"
    bad.write_text("{not json")
    with pytest.raises(MeshImportError, match="Could not read mesh file"):
        load_mesh(bad)
    listed = tmp_path / "list.json"
    listed.write_text("[]")
    with pytest.raises(MeshImportError, match="must contain a JSON object"):
        load_mesh(listed)


@pytest.mark.parametrize("split", ("half", "all"))
def test_geometry_of_a_mesh_read_from_json_equals_the_original(split):
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import vortex_case

    case, _ = vortex_case(24, split=split)
    text = json.dumps(mesh_to_dict(case.mesh))
    mesh = mesh_from_dict(json.loads(text))
    a = build_geometry(case.mesh, case)
    case.mesh = mesh
    b = build_geometry(mesh, case)
    for field in ("areas", "centers", "face_normals", "face_lengths", "owners", "neighbours", "interior_faces",
                  "gradient_sources", "gradient_neighbours", "gradient_coefficients_x", "limiter_cells",
                  "limiter_dx", "limiter_dy"):
        np.testing.assert_array_equal(np.asarray(getattr(a, field)), np.asarray(getattr(b, field)), err_msg=field)


def test_cell_face_lists_rebuild_the_stored_connectivity():
    entry = GOLDEN["valid"]["vortex12"]
    mesh = mesh_from_dict(copy.deepcopy(entry["data"]))
    ids, signs = mesh_io.cell_face_lists(mesh)
    np.testing.assert_array_equal(ids.nodes, mesh.cell_face_ids.nodes)
    np.testing.assert_array_equal(signs.nodes, mesh.cell_face_signs.nodes)
