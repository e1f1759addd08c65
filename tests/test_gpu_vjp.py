"""Reverse-mode residual product (VJP) and the wall-force functional.

The VJP is the transpose of the exact JVP (same switches), so the dot-product
identity <lambda, J v> = <J^T lambda, v> holds to rounding; the far-field
parameter gradient is checked against central differences of the residual.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(kind, n):
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, riemann_case, smooth_primitive, vortex_case, vortex_primitive

    if kind == "riemann":
        case, _ = riemann_case(n)
        P = smooth_primitive(len(case.mesh.cells), seed=3, amplitude=1.0)
    elif kind == "polygons":  # pentagons and hexagons: the any-count cell reverse
        from test_gpu_polygons import _polygon_case

        case = _polygon_case()
        P = vortex_primitive(10.0 * cell_centroids(case.mesh), mach=0.3)
        P *= 1.0 + 0.01 * np.random.default_rng(9).standard_normal(P.shape)
    else:
        case, _ = vortex_case(n, split="half")
        P = vortex_primitive(cell_centroids(case.mesh))
        P *= 1.0 + 0.01 * np.random.default_rng(9).standard_normal(P.shape)
    return case, build_geometry(case.mesh, case), P


@pytest.mark.parametrize("kind,n", (("riemann", 20), ("vortex", 16), ("polygons", 0)))
@pytest.mark.parametrize("flux", ("Rusanov", "HLLC", "Roe"))
@pytest.mark.parametrize("recon,limiter", (("First order", "Barth-Jespersen"), ("MUSCL linear", "Venkatakrishnan"),
                                           ("MUSCL linear", "Barth-Jespersen"), ("MUSCL linear", "Van Leer")))
def test_vjp_is_the_transpose_of_the_jvp(cuda_device, kind, n, flux, recon, limiter):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.model import NumericalSettings
    from oracle.oracle import Oracle

    case, g, P = _case(kind, n)
    U0 = Oracle(g).conservative(P, 1.4)
    dg = DeviceGeometry(g)
    s = NumericalSettings(flux=flux, reconstruction=recon, limiter=limiter, acceleration_x=0.2, acceleration_y=0.1)
    cfg = make_config(s)
    rng = np.random.default_rng(1)
    dev = cuda_device
    U = torch.as_tensor(U0, device=dev)
    v = torch.as_tensor(rng.standard_normal(U0.shape), device=dev)
    lam = torch.as_tensor(rng.standard_normal(U0.shape), device=dev)
    jv = torch.empty_like(U)
    vjp = torch.empty_like(U)
    stream = torch.cuda.current_stream().cuda_stream
    assert dg.lib.mcfd_jvp(dg.handle, C.byref(cfg), U.data_ptr(), v.data_ptr(), jv.data_ptr(), stream) == 0
    assert dg.lib.mcfd_vjp(dg.handle, C.byref(cfg), U.data_ptr(), lam.data_ptr(), vjp.data_ptr(), None, stream) == 0
    dg.check_status()
    a = float((lam * jv).sum())
    b = float((vjp * v).sum())
    scale = float((lam.abs() * jv.abs()).sum())
    assert abs(a - b) <= 1e-12 * scale, (a, b)


@pytest.mark.parametrize("flux", ("Rusanov", "HLLC", "Roe"))
def test_far_field_parameter_gradient(cuda_device, flux):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.geometry import build_geometry
    from oracle.oracle import Oracle

    case, g, P = _case("riemann", 16)
    s = case.numerics
    s.flux, s.reconstruction, s.limiter = flux, "MUSCL linear", "Venkatakrishnan"
    cfg = make_config(s)
    dev = cuda_device
    U0 = Oracle(g).conservative(P, 1.4)
    U = torch.as_tensor(U0, device=dev)
    lam = torch.as_tensor(np.random.default_rng(2).standard_normal(U0.shape), device=dev)
    dg = DeviceGeometry(g)
    nf = len(g.far_field_faces)
    ubar = torch.empty_like(U)
    fbar = torch.empty(nf, 4, dtype=torch.float64, device=dev)
    assert dg.lib.mcfd_vjp(dg.handle, C.byref(cfg), U.data_ptr(), lam.data_ptr(), ubar.data_ptr(), fbar.data_ptr(),
                           torch.cuda.current_stream().cuda_stream) == 0
    dg.check_status()
    # gradient with respect to the "right" patch's far-field state, by patch
    right = next(c for c in case.boundary_conditions if c.patch_name == "right")
    base = dict(right.values)
    mask = np.isin(g.far_field_faces, np.asarray(next(p for p in case.mesh.patches if p.name == "right").face_ids))
    grad = fbar.cpu().numpy()[mask].sum(axis=0)
    keys = ("density", "velocity_x", "velocity_y", "pressure")
    for k, key in enumerate(keys):
        h = 1e-6 * max(1.0, abs(base[key]))
        vals = []
        for sign in (1, -1):
            right.values = dict(base, **{key: base[key] + sign * h})
            gk = build_geometry(case.mesh, case)
            R = DeviceGeometry(gk).residual(U, cfg)
            vals.append(float((lam * R).sum()))
        right.values = dict(base)
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - grad[k]) <= 1e-6 * max(1.0, abs(fd)), (key, fd, grad[k])


def test_wall_force_and_its_gradient(cuda_device):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from oracle.oracle import Oracle

    case, g, P = _case("riemann", 16)
    cfg = make_config(case.numerics)
    dg = DeviceGeometry(g)
    U0 = Oracle(g).conservative(P, 1.4)
    U = torch.as_tensor(U0, device=cuda_device)
    J = (C.c_double * 1)()
    dJ = torch.empty_like(U)
    assert dg.lib.mcfd_wall_force(dg.handle, C.byref(cfg), U.data_ptr(), 0.3, 0.8, J, dJ.data_ptr(),
                                  torch.cuda.current_stream().cuda_stream) == 0
    wf = np.asarray(g.wall_faces)
    o = np.asarray(g.owners)[wf]
    n = np.asarray(g.face_normals)[wf]
    ref = float(np.sum(P[o, 3] * (n[:, 0] * 0.3 + n[:, 1] * 0.8) * np.asarray(g.face_lengths)[wf]))
    assert abs(J[0] - ref) <= 1e-13 * abs(ref)
    # directional derivative against central differences
    d = np.random.default_rng(4).standard_normal(U0.shape) * 1e-3
    vals = []
    for sign in (1, -1):
        Jp = (C.c_double * 1)()
        Ut = torch.as_tensor(U0 + sign * 1e-4 * d, device=cuda_device)
        dg.lib.mcfd_wall_force(dg.handle, C.byref(cfg), Ut.data_ptr(), 0.3, 0.8, Jp, None,
                               torch.cuda.current_stream().cuda_stream)
        vals.append(Jp[0])
    fd = (vals[0] - vals[1]) / (2e-4)
    assert abs(fd - float((dJ.cpu().numpy() * d).sum())) <= 1e-8 * max(1.0, abs(fd))
