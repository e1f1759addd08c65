"""The smooth Venkatakrishnan limiter (the published form with the constant K,
an extension with no counterpart in the reference) on the GPU: forward
kernels against the oracle's C restatement in every kernel variant, the
exact JVP against central differences and the reverse mode against the JVP
(transpose) and torch autograd of the torch-op residual."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _case(kind="periodic", flux="HLLC", k=5.0):
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import riemann_case, periodic_case, smooth_primitive

    if kind == "periodic":
        case = periodic_case(20, 16, split="half", jitter=0.2, seed=5)
    else:
        case, _ = riemann_case(16)
    s = case.numerics
    s.flux, s.reconstruction, s.limiter = flux, "MUSCL linear", "Venkatakrishnan K"
    s.venkatakrishnan_k = k
    g = build_geometry(case.mesh, case)
    return s, g, smooth_primitive(len(g.areas), seed=3, amplitude=0.2)


@pytest.mark.parametrize("kind", ("periodic", "riemann"))
@pytest.mark.parametrize("flux", ("Rusanov", "HLLC", "Roe"))
def test_residual_matches_the_oracle_in_every_variant(cuda_device, kind, flux):
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from oracle.oracle import Oracle

    s, g, P = _case(kind, flux)
    orc = Oracle(g)
    U0 = orc.conservative(P, s.gamma)
    ref = orc.residual(U0, s)
    dg = DeviceGeometry(g)
    U = torch.as_tensor(U0, device=cuda_device)
    for mode in ("exact", "fast", "fma"):
        R = dg.residual(U, make_config(s, mode)).cpu().numpy()
        dg.check_status()
        if mode == "fma":
            assert np.abs(R - ref).max() <= 1e-12 * np.abs(ref).max(), mode
        elif kind == "periodic":
            np.testing.assert_array_equal(R, ref, err_msg=mode)
        else:  # far field: pow() differs in the last place between libm and CUDA
            assert np.abs(R - ref).max() <= 1e-14 * np.abs(ref).max(), mode


def test_rk3_steps_match_the_oracle_bit_for_bit(cuda_device):
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.solver import run_explicit
    from oracle.oracle import Oracle

    s, g, P = _case("periodic", "HLLC")
    s.time_integration, s.cfl, s.end_time, s.max_iterations, s.residual_tolerance = "Explicit RK3", 0.8, 1e30, 20, 1e-300
    orc = Oracle(g)
    U0 = orc.conservative(P, s.gamma)
    ref, t = orc.solve(U0, s, 20)
    dg = DeviceGeometry(g)
    U = torch.as_tensor(U0, device=cuda_device)
    for mode in ("exact", "fast"):
        U.copy_(torch.as_tensor(U0, device=cuda_device))
        result = run_explicit(dg, s, U, mode=mode, final_residual=False)
        assert result.steps == 20 and result.time == t
        np.testing.assert_array_equal(U.cpu().numpy(), ref, err_msg=mode)


@pytest.mark.parametrize("flux", ("Rusanov", "HLLC", "Roe"))
def test_jvp_vjp_and_torch_autograd(cuda_device, flux):
    from meshcfd_gb300.adjoint import ResidualFunction
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from oracle.oracle import Oracle
    from oracle.torch_residual import TorchResidual

    s, g, P = _case("riemann", flux)
    orc = Oracle(g)
    U0 = orc.conservative(P, s.gamma)
    rng = np.random.default_rng(5)
    lam = rng.standard_normal(U0.shape)
    v = rng.standard_normal(U0.shape) * np.abs(U0)
    dg = DeviceGeometry(g)
    cfg = make_config(s)
    stream = torch.cuda.current_stream().cuda_stream
    U = torch.as_tensor(U0, device=cuda_device)
    jv = torch.empty_like(U)
    v_d = torch.as_tensor(v, device=cuda_device)
    assert dg.lib.mcfd_jvp(dg.handle, C.byref(cfg), U.data_ptr(), v_d.data_ptr(), jv.data_ptr(), stream) == 0
    Ug = U.clone().requires_grad_(True)
    (ResidualFunction.apply(Ug, dg, cfg) * torch.as_tensor(lam, device=cuda_device)).sum().backward()
    dg.check_status()
    # transpose: <lam, J v> = <J^T lam, v>
    a, b = float((torch.as_tensor(lam, device=cuda_device) * jv).sum()), float((Ug.grad * torch.as_tensor(v, device=cuda_device)).sum())
    assert abs(a - b) <= 1e-12 * float((np.abs(lam) * np.abs(jv.cpu().numpy())).sum())
    # JVP against central differences of the residual (smooth limiter)
    h = 1e-7
    fd = (orc.residual(U0 + h * v, s) - orc.residual(U0 - h * v, s)) / (2 * h)
    assert np.abs(jv.cpu().numpy() - fd).max() <= 1e-6 * np.abs(fd).max()
    # reverse mode against torch autograd of the torch-op residual
    ref = TorchResidual(g, s)
    Ut = torch.as_tensor(U0).requires_grad_(True)
    (torch.as_tensor(lam) * ref(Ut)).sum().backward()
    gu = Ut.grad.numpy()
    assert np.abs(Ug.grad.cpu().numpy() - gu).max() <= 1e-11 * np.abs(gu).max()


def test_refused_with_parabolic_reconstruction(cuda_device):
    from meshcfd_gb300.device import DeviceGeometry, make_config

    s, g, P = _case()
    s.reconstruction = "MUSCL parabolic"
    dg = DeviceGeometry(g)
    cfg = make_config(s)
    U = torch.ones(dg.n_cells, 4, dtype=torch.float64, device=cuda_device)
    R = torch.empty_like(U)
    assert dg.lib.mcfd_residual(dg.handle, C.byref(cfg), U.data_ptr(), R.data_ptr(),
                                torch.cuda.current_stream().cuda_stream) == 3  # MCFD_E_UNSUPPORTED
