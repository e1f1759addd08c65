"""The geometry build with its numeric loops on the device
(geometry_device.DeviceGeometryBuilder: cell centroids and areas, face
centres / normals / lengths, least-squares gradient offsets and
coefficients, limiter offsets in the library's kernels) gives the host
build's arrays bit for bit, on periodic, wall / far-field / outlet, curved
(O-grid), randomly numbered, all-triangle and parabolic meshes, and reports
the host build's errors."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _case(name):
    from meshcfd_gb300.meshes import (bump_case, ogrid_case, periodic_case, permute_mesh, riemann_case,
                                      vortex_case)

    if name == "vortex":
        return vortex_case(64, split="half")[0]
    if name == "vortex_parabolic":
        case = vortex_case(32, split="half")[0]
        case.numerics.reconstruction = "MUSCL parabolic"
        return case
    if name == "bump":
        return bump_case(48, 24)[0]
    if name == "ogrid":
        return ogrid_case(64, 32)[0]
    if name == "riemann":
        return riemann_case(32)[0]
    case = periodic_case(40, 40, split="all", jitter=0.2, seed=5)
    rng = np.random.default_rng(1)
    case.mesh = permute_mesh(case.mesh, rng.permutation(len(case.mesh.cells)), rng.permutation(len(case.mesh.faces)))
    return case


@pytest.mark.parametrize("name", ("vortex", "vortex_parabolic", "bump", "ogrid", "riemann", "permuted"))
def test_device_geometry_build_equals_the_host_build(cuda_device, name):
    from dataclasses import fields

    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.geometry_device import DeviceGeometryBuilder

    case = _case(name)
    host = build_geometry(case.mesh, case)
    dev = build_geometry(case.mesh, case, host=DeviceGeometryBuilder(cuda_device))
    compared = 0
    for f in fields(host):
        a, b = getattr(host, f.name), getattr(dev, f.name)
        if isinstance(a, np.ndarray):
            assert a.shape == b.shape and a.dtype == b.dtype, f.name
            np.testing.assert_array_equal(b, a, err_msg=f.name)
            compared += 1
    assert compared >= 30


def test_device_geometry_build_reports_a_degenerate_cell(cuda_device):
    from dataclasses import replace

    from meshcfd_gb300.errors import SolverError
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.geometry_device import DeviceGeometryBuilder
    from meshcfd_gb300.meshes import vortex_case

    case = vortex_case(8, split="none")[0]
    pts = np.array(case.mesh.points, dtype=float, copy=True)
    nodes = np.asarray(case.mesh.cells.nodes)
    off = np.asarray(case.mesh.cells.offsets)
    pts[nodes[off[5]:off[6]]] = pts[nodes[off[5]]]  # cell 5 collapsed to a point
    case.mesh = replace(case.mesh, points=pts)
    with pytest.raises(SolverError) as host_error:
        build_geometry(case.mesh, case)
    with pytest.raises(SolverError) as dev_error:
        build_geometry(case.mesh, case, host=DeviceGeometryBuilder(cuda_device))
    assert str(dev_error.value) == str(host_error.value)
