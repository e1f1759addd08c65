"""Exact Jacobian-vector product (forward mode) on the GPU.

The reference has no exact Jacobian; its implicit operator is a finite
difference (solver.py:1532-1567).  Checks: central differences of the GPU
residual (step 1e-6 relative to the state), the exact implicit operator
against the finite-difference one, and an implicit solve with the exact
Jacobian against the reference's converged states.
"""

import ctypes as C

import numpy as np
import pytest

from conftest import load_fixture, solve_settings

pytestmark = pytest.mark.gpu


def _case(kind, n):
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, riemann_case, smooth_primitive, vortex_case, vortex_primitive

    if kind == "riemann":
        case, _ = riemann_case(n)
        P = smooth_primitive(len(case.mesh.cells), seed=3, amplitude=1.0)
    else:
        case, _ = vortex_case(n, split="half")
        # the exact vortex has a uniform free stream where neighbouring states
        # tie exactly (limiter and wave-speed kinks); perturb it so that no
        # switch sits within the finite-difference step
        P = vortex_primitive(cell_centroids(case.mesh))
        P *= 1.0 + 0.01 * np.random.default_rng(9).standard_normal(P.shape)
    return case, build_geometry(case.mesh, case), P


@pytest.mark.parametrize("kind,n", (("riemann", 24), ("vortex", 20)))
@pytest.mark.parametrize("flux", ("Rusanov", "HLLC", "Roe"))
@pytest.mark.parametrize("recon,limiter", (("First order", "Barth-Jespersen"), ("MUSCL linear", "Venkatakrishnan"),
                                           ("MUSCL linear", "Van Leer")))
def test_jvp_matches_central_differences(cuda_device, kind, n, flux, recon, limiter):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.model import NumericalSettings
    from oracle.oracle import Oracle

    case, g, P = _case(kind, n)
    orc = Oracle(g)
    U0 = orc.conservative(P, 1.4)
    dg = DeviceGeometry(g)
    s = NumericalSettings(flux=flux, reconstruction=recon, limiter=limiter, acceleration_x=0.1, acceleration_y=-0.05)
    cfg = make_config(s)
    rng = np.random.default_rng(5)
    dU = rng.standard_normal(U0.shape) * np.abs(U0).max(axis=0)
    U = torch.as_tensor(U0, device=cuda_device)
    d = torch.as_tensor(dU, device=cuda_device)
    out = torch.empty_like(U)
    assert dg.lib.mcfd_jvp(dg.handle, C.byref(cfg), U.data_ptr(), d.data_ptr(), out.data_ptr(),
                           torch.cuda.current_stream().cuda_stream) == 0
    dg.check_status()
    h = 1e-6 if recon == "First order" else 1e-8
    Rp = dg.residual(U + h * d, cfg)
    Rm = dg.residual(U - h * d, cfg)
    fd = ((Rp - Rm) / (2 * h)).cpu().numpy()
    jv = out.cpu().numpy()
    tol = 1e-5 if recon == "First order" else 1e-4
    assert np.abs(jv - fd).max() <= tol * np.abs(fd).max(), np.abs(jv - fd).max() / np.abs(fd).max()


@pytest.mark.parametrize("name", ("implicit_channel.npz", "implicit_periodic.npz"))
def test_exact_operator_matches_finite_difference_operator(cuda_device, name):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config

    data, geom = load_fixture(name)
    s = solve_settings(data)
    dg = DeviceGeometry(geom)
    cfg = make_config(s)
    U = torch.as_tensor(data["U"], device=cuda_device)
    dt = torch.as_tensor(data["dt_cells"], device=cuda_device)
    scales = (C.c_double * 4)(*data["scales"])
    stream = torch.cuda.current_stream().cuda_stream
    assert dg.lib.mcfd_implicit_prepare(dg.handle, C.byref(cfg), U.data_ptr(), dt.data_ptr(), 1, scales, stream) == 0
    v = torch.as_tensor(data["v"], device=cuda_device)
    fd = torch.empty_like(v)
    ex = torch.empty_like(v)
    assert dg.lib.mcfd_implicit_matvec(dg.handle, v.data_ptr(), fd.data_ptr(), stream) == 0
    assert dg.lib.mcfd_implicit_set_jacobian(dg.handle, 1) == 0
    assert dg.lib.mcfd_implicit_matvec(dg.handle, v.data_ptr(), ex.data_ptr(), stream) == 0
    dg.check_status()
    a, b = ex.cpu().numpy(), fd.cpu().numpy()
    assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()
    assert np.abs(a - data["operator_v"]).max() <= 1e-6 * np.abs(data["operator_v"]).max()


@pytest.mark.parametrize("name", ("implicit_channel.npz", "implicit_periodic.npz"))
def test_implicit_solve_with_exact_jacobian(cuda_device, name):
    import torch
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.implicit import run_implicit
    from oracle.oracle import Oracle

    data, geom = load_fixture(name)
    s = solve_settings(data)
    dg = DeviceGeometry(geom)
    assert dg.lib.mcfd_implicit_set_jacobian(dg.handle, 1) == 0
    U = torch.as_tensor(data["U"], device=cuda_device)
    time, steps, _ = run_implicit(dg, s, U, max_steps=int(data["steps"]))
    P = Oracle(geom).primitive(U.cpu().numpy(), s.gamma)
    ref = data["P_final"]
    assert np.abs(P - ref).max() <= 1e-7 * np.abs(ref).max()
