import sys
import types
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
for p in (str(ROOT), str(GOLDEN)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_fixture(name):
    """Load a golden .npz as a dict (arrays) with a geometry namespace."""
    data = dict(np.load(GOLDEN / name, allow_pickle=False))
    patches = ([], [], [])
    if "bcp_kind" in data:
        off = data["bcp_offsets"]
        for k, (kind, pname, v) in enumerate(zip(data["bcp_kind"], data["bcp_names"], data["bcp_values"])):
            faces = data["bcp_faces"][off[k]:off[k + 1]]
            if kind == 0:
                b = types.SimpleNamespace(faces=faces, total_pressure=float(v[0]), total_temperature=float(v[1]),
                                          direction=np.asarray(v[2:4]), patch_name=str(pname))
            elif kind == 1:
                b = types.SimpleNamespace(faces=faces, mass_flow=float(v[0]), total_temperature=float(v[1]),
                                          direction=np.asarray(v[2:4]), patch_name=str(pname))
            else:
                b = types.SimpleNamespace(faces=faces, mass_flow=float(v[0]), patch_name=str(pname))
            patches[int(kind)].append(b)
    walls = []
    if "wt_offsets" in data:
        off = data["wt_offsets"]
        for k in range(len(off) - 1):
            walls.append(types.SimpleNamespace(faces=data["wt_faces"][off[k]:off[k + 1]],
                                               condition=str(data["wt_condition"][k]), value=float(data["wt_value"][k]),
                                               patch_name=str(data["wt_names"][k]),
                                               mechanical_condition=str(data["wt_mechanical"][k])))
    kinds = {}
    if "patch_kind_ids" in data:
        kinds = {int(i): str(n) for i, n in zip(data["patch_kind_ids"], data["patch_kind_names"])}
    geom = types.SimpleNamespace(
        **{k[5:]: v for k, v in data.items() if k.startswith("geom_")},
        pressure_inlets=tuple(patches[0]), mass_flow_inlets=tuple(patches[1]), mass_flow_outlets=tuple(patches[2]),
        wall_thermal_boundaries=tuple(walls), patch_kinds=kinds,
    )
    return data, geom


def viscous_settings_for(key, data):
    """Settings of a viscous fixture key R|flux|recon|limiter|force|model."""
    s = settings_for("|".join(key.split("|")[:5]))
    s.viscosity_model = key.split("|")[5]
    s.dynamic_viscosity = float(data["dynamic_viscosity"])
    return s


def fixture_mesh(data):
    from meshcfd_gb300.meshes import CellArray
    from meshcfd_gb300.model import FiniteVolumeMesh

    return FiniteVolumeMesh(
        points=data["mesh_points"], cells=CellArray(data["mesh_cell_offsets"], data["mesh_cell_nodes"]),
        faces=data["mesh_faces"], face_owners=data["mesh_face_owners"],
        face_neighbours=data["mesh_face_neighbours"], face_patch_ids=data["mesh_face_patch_ids"], patches=(),
    )


def residual_keys(data):
    return sorted(k for k in data if k.startswith("R|"))


def settings_for(key):
    from meshcfd_gb300.model import NumericalSettings

    _, flux, recon, limiter, force = key.split("|")
    s = NumericalSettings(flux=flux, reconstruction=recon, limiter=limiter)
    if force == "1":
        s.acceleration_x, s.acceleration_y = 0.3, -0.2
    return s


def solve_settings(data):
    from meshcfd_gb300.model import NumericalSettings

    s = NumericalSettings()
    for k, v in data.items():
        if k.startswith("set|"):
            setattr(s, k[4:], v.item() if v.dtype.kind != "U" else str(v))
    s.end_time = 1.0e30
    s.max_iterations = int(data["steps"])
    s.residual_tolerance = 1e-300
    return s


@pytest.fixture(scope="session")
def cuda_device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)
