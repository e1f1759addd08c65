"""Reverse mode on the GPU against torch autograd of the FP64 PyTorch-op
residual, and the checkpointed RK3 adjoint of the wall force against both
torch autograd of the unrolled time march and central differences."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _state_case(kind, n):
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, riemann_case, smooth_primitive, vortex_case, vortex_primitive

    if kind == "riemann":
        case, _ = riemann_case(n)
        P = smooth_primitive(len(case.mesh.cells), seed=3, amplitude=1.0)
    else:
        case, _ = vortex_case(n, split="half")
        P = vortex_primitive(cell_centroids(case.mesh))
        P *= 1.0 + 0.01 * np.random.default_rng(9).standard_normal(P.shape)
    return case, build_geometry(case.mesh, case), P


@pytest.mark.parametrize("kind,n", (("riemann", 20), ("vortex", 16)))
@pytest.mark.parametrize("flux", ("Rusanov", "HLLC", "Roe"))
@pytest.mark.parametrize("recon,limiter", (("First order", "Barth-Jespersen"), ("MUSCL linear", "Venkatakrishnan"),
                                           ("MUSCL linear", "Minmod"), ("MUSCL linear", "Van Leer")))
def test_vjp_matches_torch_autograd(cuda_device, kind, n, flux, recon, limiter):
    from meshcfd_gb300.adjoint import ResidualFunction
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.model import NumericalSettings
    from oracle.oracle import Oracle
    from oracle.torch_residual import TorchResidual

    case, g, P = _state_case(kind, n)
    U0 = Oracle(g).conservative(P, 1.4)
    s = NumericalSettings(flux=flux, reconstruction=recon, limiter=limiter, acceleration_x=0.2, acceleration_y=0.1)
    lam = np.random.default_rng(5).standard_normal(U0.shape)

    ref = TorchResidual(g, s)
    Ut = torch.as_tensor(U0).requires_grad_(True)
    far = ref.far_states.clone().requires_grad_(True)
    (torch.as_tensor(lam) * ref(Ut, far)).sum().backward()

    dg = DeviceGeometry(g)
    cfg = make_config(s)
    U = torch.as_tensor(U0, device=cuda_device).requires_grad_(True)
    R = ResidualFunction.apply(U, dg, cfg)
    (ubar,) = torch.autograd.grad(R, U, torch.as_tensor(lam, device=cuda_device))
    fbar = torch.zeros(max(dg.n_far_field, 1), 4, dtype=torch.float64, device=cuda_device)
    ubar2 = torch.empty_like(ubar)
    lam_d = torch.as_tensor(lam, device=cuda_device)
    assert dg.lib.mcfd_vjp(dg.handle, C.byref(cfg), U.data_ptr(), lam_d.data_ptr(),
                           ubar2.data_ptr(), fbar.data_ptr(), torch.cuda.current_stream().cuda_stream) == 0
    dg.check_status()
    assert torch.equal(ubar, ubar2)
    gu = Ut.grad.numpy()
    err = np.abs(ubar.cpu().numpy() - gu).max()
    assert err <= 1e-11 * np.abs(gu).max(), err
    if dg.n_far_field:
        gf = far.grad.numpy()
        err = np.abs(fbar.cpu().numpy() - gf).max()
        assert err <= 1e-11 * max(np.abs(gf).max(), 1e-300), err


# ----------------------------------------------------------- RK3 adjoint


def _ogrid(inflow=None, n_theta=32, n_r=8):
    """Small O-grid around a cylinder (far field one radius from the wall, so
    the inflow reaches the wall force within the run); initial state = inflow
    + a fixed seeded 10 % perturbation, large enough that no limiter or flux
    switch lies within the finite-difference steps."""
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import ogrid_case

    case, P = ogrid_case(n_theta, n_r, half_width=1.0, seed=2, mach=0.3)
    far = next(c for c in case.boundary_conditions if c.kind == "Far Field")
    keys = ("density", "velocity_x", "velocity_y", "pressure")
    base = np.array([far.values[k] for k in keys])
    if inflow is not None:
        far.values = dict(zip(keys, map(float, inflow)))
        base = np.asarray(inflow, dtype=float)
    rng = np.random.default_rng(11)
    scale = np.array([1.0, 0.3, 0.3, 1.0])
    P0 = base + 0.1 * scale * rng.standard_normal(P.shape)
    return case, build_geometry(case.mesh, case), P0, base


def _dt(g, case, P0):
    from oracle.oracle import Oracle

    return 0.5 * float(Oracle(g).stable_time_steps(P0, case.numerics).min())


STEPS, EVERY = 20, 6
# central differences with step 1e-6 against the adjoint gradient
TOL_FD = 1e-6


def test_rk3_adjoint_matches_unrolled_torch_autograd(cuda_device):
    from meshcfd_gb300.adjoint import WallForceAdjoint
    from meshcfd_gb300.device import DeviceGeometry
    from oracle.oracle import Oracle
    from oracle.torch_residual import TorchResidual, primitive

    case, g, P0, _ = _ogrid()
    U0 = Oracle(g).conservative(P0, 1.4)
    dt = _dt(g, case, P0)
    d = (0.6, 0.8)

    adj = WallForceAdjoint(DeviceGeometry(g), case.numerics, dt, direction=d, checkpoint_every=EVERY)
    J, lam0, far_grad = adj.gradient(torch.as_tensor(U0, device=cuda_device), STEPS)

    ref = TorchResidual(g, case.numerics)
    Ut = torch.as_tensor(U0).requires_grad_(True)
    far = ref.far_states.clone().requires_grad_(True)
    U = Ut
    for _ in range(STEPS):
        U1 = U + dt * ref(U, far)
        U2 = 0.75 * U + 0.25 * (U1 + dt * ref(U1, far))
        U = (1.0 / 3.0) * U + (2.0 / 3.0) * (U2 + dt * ref(U2, far))
    wf = torch.as_tensor(np.asarray(g.wall_faces))
    own = torch.as_tensor(np.asarray(g.owners))[wf]
    nrm = torch.as_tensor(np.asarray(g.face_normals).reshape(-1, 2))[wf]
    length = torch.as_tensor(np.asarray(g.face_lengths))[wf]
    Jt = (primitive(U, 1.4)[own, 3] * (nrm[:, 0] * d[0] + nrm[:, 1] * d[1]) * length).sum()
    Jt.backward()

    assert abs(J - float(Jt)) <= 1e-12 * abs(float(Jt))
    gu = Ut.grad.numpy()
    assert np.abs(lam0.cpu().numpy() - gu).max() <= 1e-9 * np.abs(gu).max()
    gf = far.grad.numpy()
    assert np.abs(far_grad[: len(gf)] - gf).max() <= 1e-9 * np.abs(gf).max()


def test_rk3_adjoint_inflow_gradient_matches_finite_differences(cuda_device):
    """dJ/d(inflow rho, u, v, p): far-field faces plus the initial state."""
    from meshcfd_gb300.adjoint import WallForceAdjoint, conservative_jacobian_T
    from meshcfd_gb300.device import DeviceGeometry
    from oracle.oracle import Oracle

    case, g, P0, base = _ogrid()
    dt = _dt(g, case, P0)

    def run(inflow, grad=False):
        c, gk, Pk, _ = _ogrid(inflow)
        adj = WallForceAdjoint(DeviceGeometry(gk), c.numerics, dt, direction=(1.0, 0.0), checkpoint_every=EVERY)
        U0 = torch.as_tensor(Oracle(gk).conservative(Pk, 1.4), device=cuda_device)
        if not grad:
            return adj.functional(adj.forward(U0, STEPS))[0]
        J, lam0, far_grad = adj.gradient(U0, STEPS)
        total = far_grad[: len(gk.far_field_faces)].sum(0)
        total += conservative_jacobian_T(Pk, lam0.cpu().numpy(), 1.4).sum(0)
        return J, total

    J, grad = run(base, grad=True)
    for k in range(4):
        h = 1e-6 * max(1.0, abs(base[k]))
        e = np.zeros(4)
        e[k] = h
        fd = (run(base + e) - run(base - e)) / (2 * h)
        assert abs(fd - grad[k]) <= TOL_FD * max(abs(fd), 1e-3 * abs(J)), (k, fd, grad[k])


@pytest.mark.parametrize("limiter,h", (("Venkatakrishnan K", 1e-6), ("Venkatakrishnan", 1e-7)))
def test_rk3_adjoint_initial_state_direction_matches_finite_differences(cuda_device, limiter, h):
    """Initial-state direction (each cell's state scaled by its own size).
    With the smooth limiter (K = 5) from a smooth disturbance, the central
    difference with step 1e-6 is within 1e-6 of the adjoint.  With the reference's capped form the
    function is only piecewise smooth and strongly curved on this rough
    state: the step-1e-6 difference carries a truncation error of 1.8e-6
    (measured: it falls as h^2 to 3.7e-9 at 1e-7), so that check uses 1e-7."""
    from meshcfd_gb300.adjoint import WallForceAdjoint
    from meshcfd_gb300.device import DeviceGeometry
    from oracle.oracle import Oracle

    case, g, P0, base = _ogrid()
    case.numerics.limiter = limiter
    if limiter == "Venkatakrishnan K":  # the smooth limiter on a smooth disturbance
        centers = np.asarray(g.centers).reshape(-1, 2)
        P0 = base * (1.0 + _smooth_perturbation(centers, seed=11, amplitude=0.1) * np.array([1.0, 0.3, 0.3, 1.0]))
    dt = _dt(g, case, P0)
    U0 = Oracle(g).conservative(P0, 1.4)
    adj = WallForceAdjoint(DeviceGeometry(g), case.numerics, dt, direction=(0.0, 1.0), checkpoint_every=EVERY)
    _, lam0, _ = adj.gradient(torch.as_tensor(U0, device=cuda_device), STEPS)
    v = np.random.default_rng(12).standard_normal(U0.shape) * np.abs(U0)
    vals = [adj.functional(adj.forward(torch.as_tensor(U0 + sgn * h * v, device=cuda_device), STEPS))[0]
            for sgn in (1, -1)]
    fd = (vals[0] - vals[1]) / (2 * h)
    an = float((lam0.cpu().numpy() * v).sum())
    assert abs(fd - an) <= TOL_FD * max(abs(fd), 1e-12), (fd, an)


def test_checkpoint_interval_does_not_change_the_gradient(cuda_device):
    from meshcfd_gb300.adjoint import WallForceAdjoint, WallForceFunction
    from meshcfd_gb300.device import DeviceGeometry
    from oracle.oracle import Oracle

    case, g, P0, _ = _ogrid()
    dt = _dt(g, case, P0)
    U0 = torch.as_tensor(Oracle(g).conservative(P0, 1.4), device=cuda_device)
    dg = DeviceGeometry(g)
    lams = []
    for every in (1, 3, 100):
        adj = WallForceAdjoint(dg, case.numerics, dt, checkpoint_every=every)
        lams.append(adj.gradient(U0, STEPS)[1])
    assert torch.equal(lams[0], lams[1]) and torch.equal(lams[0], lams[2])
    # the same adjoint through torch autograd
    Ux = U0.clone().requires_grad_(True)
    J = WallForceFunction.apply(Ux, WallForceAdjoint(dg, case.numerics, dt, checkpoint_every=4), STEPS)
    (g0,) = torch.autograd.grad(2.0 * J, Ux)
    assert torch.equal(g0, 2.0 * lams[0])


def test_recorded_step_and_vjp_at_match_plain_calls(cuda_device):
    """mcfd_explicit_step_record advances exactly like mcfd_explicit_step and
    records each stage's primitive and face states; mcfd_vjp_at at those
    states equals mcfd_vjp bit for bit."""
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from oracle.oracle import Oracle

    case, g, P0, _ = _ogrid()
    U0 = torch.as_tensor(Oracle(g).conservative(P0, 1.4), device=cuda_device)
    dg = DeviceGeometry(g)
    cfg = make_config(case.numerics)
    dt = torch.full((1,), _dt(g, case, P0), dtype=torch.float64, device=cuda_device)
    n, nl = dg.n_cells, int(dg.info.n_limiter)
    Ps = [torch.empty(n, 4, dtype=torch.float64, device=cuda_device) for _ in range(3)]
    Rs = [torch.empty(nl, 4, dtype=torch.float64, device=cuda_device) for _ in range(3)]
    Ua, Ub = U0.clone(), U0.clone()
    dg.explicit_step(Ua, cfg, 2, dt)
    stream = torch.cuda.current_stream().cuda_stream
    assert dg.lib.mcfd_explicit_step_record(dg.handle, C.byref(cfg), 2, Ub.data_ptr(), dt.data_ptr(), 0,
                                            (C.c_void_p * 3)(*[t.data_ptr() for t in Ps]),
                                            (C.c_void_p * 3)(*[t.data_ptr() for t in Rs]), 3, stream) == 0
    dg.check_status()
    assert torch.equal(Ua, Ub)
    assert torch.equal(Ps[0], dg.primitive(U0, cfg))
    lam = torch.as_tensor(np.random.default_rng(3).standard_normal((n, 4)), device=cuda_device)
    a, b = torch.empty_like(lam), torch.empty_like(lam)
    assert dg.lib.mcfd_vjp(dg.handle, C.byref(cfg), U0.data_ptr(), lam.data_ptr(), a.data_ptr(), None, stream) == 0
    assert dg.lib.mcfd_vjp_at(dg.handle, C.byref(cfg), U0.data_ptr(), Ps[0].data_ptr(), Rs[0].data_ptr(),
                              lam.data_ptr(), b.data_ptr(), None, stream) == 0
    dg.check_status()
    assert torch.equal(a, b)
    c = torch.empty_like(lam)  # the recorded primitive suffices: no conservative state
    assert dg.lib.mcfd_vjp_at(dg.handle, C.byref(cfg), None, Ps[0].data_ptr(), Rs[0].data_ptr(),
                              lam.data_ptr(), c.data_ptr(), None, stream) == 0
    assert torch.equal(a, c)


def _smooth_perturbation(centers, seed, amplitude=0.1):
    """A seeded sum of a few long-wave sine modes (wavelengths 2-8 units) per
    variable, scaled to ``amplitude`` at most: a smooth initial disturbance."""
    rng = np.random.default_rng(seed)
    out = np.zeros((len(centers), 4))
    for v in range(4):
        for _ in range(4):
            k = 2.0 * np.pi / rng.uniform(2.0, 8.0, size=2) * rng.choice((-1.0, 1.0), size=2)
            out[:, v] += rng.uniform(0.5, 1.0) * np.sin(centers @ k + rng.uniform(0.0, 2.0 * np.pi))
    return amplitude * out / np.abs(out).max(axis=0)


def _blob_direction(centers, U0, center=(-1.5, 0.2), width=0.5):
    """A smooth, localised initial-state direction: a Gaussian blob upstream
    of the cylinder in every variable (scaled by the state's own size)."""
    r2 = ((centers - np.asarray(center)) ** 2).sum(axis=1)
    return np.exp(-r2 / width**2)[:, None] * np.abs(U0) * np.array([1.0, 0.5, -0.7, 0.8])


@pytest.mark.parametrize("limiter", ("Venkatakrishnan", "Venkatakrishnan K"))
def test_full_size_ogrid_adjoint_matches_finite_differences(cuda_device, limiter):
    """The differentiation configuration at its full size: the 1024 x 512
    O-grid around the cylinder (half width 10, seed 2, Mach 0.3), HLLC,
    MUSCL linear with the reference's Venkatakrishnan limiter or the smooth
    form (K = 5), 400 RK3 steps of a fixed time step with checkpoints every
    20 steps, from the inflow state plus the seeded 10 % perturbation.  The
    adjoint gradient of the x wall force in a smooth, localised
    initial-state direction against central differences with step 1e-6,
    within 1e-6 (measured: 7e-9 and 3e-9).

    A direction that moves every cell's state independently is not a usable
    finite-difference probe at this size: over 400 steps and half a million
    cells a step of 1e-6 crosses flux and limiter switches somewhere, and
    the derivative in such a direction is a sum of terms of both signs much
    smaller than its parts, so the quotient's error relative to it grows
    (measured 1e-4 to 3e-4 at step 1e-6, falling to 9e-9 at step 1e-9 as the
    crossings become rare).  The inflow gradient of this configuration is
    identically zero: in 400 steps of the wall-limited time step a signal
    from the far field crosses a small fraction of the 9.5 units to the
    wall, so the inflow check above runs on the small box."""
    from meshcfd_gb300.adjoint import WallForceAdjoint
    from meshcfd_gb300.device import DeviceGeometry, primitive_to_conservative
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import ogrid_case

    case, P = ogrid_case(1024, 512, seed=2, mach=0.3)
    case.numerics.limiter = limiter
    case.numerics.venkatakrishnan_k = 5.0
    g = build_geometry(case.mesh, case)
    assert len(g.areas) == 524288
    rng = np.random.default_rng(11)
    P0 = P + 0.1 * np.array([1.0, 0.3, 0.3, 1.0]) * rng.standard_normal(P.shape)
    U0 = primitive_to_conservative(P0, 1.4)
    dg = DeviceGeometry(g)
    dt = _dt(g, case, P0)
    adj = WallForceAdjoint(dg, case.numerics, dt, direction=(1.0, 0.0), checkpoint_every=20)
    steps = 400
    _, lam0, _ = adj.gradient(torch.as_tensor(U0, device=cuda_device), steps)
    assert np.all(np.isfinite(lam0.cpu().numpy()))
    v = _blob_direction(np.asarray(g.centers).reshape(-1, 2), U0)
    h = 1e-6
    vals = [adj.functional(adj.forward(torch.as_tensor(U0 + sgn * h * v, device=cuda_device), steps))[0]
            for sgn in (1, -1)]
    dg.check_status()
    fd = (vals[0] - vals[1]) / (2 * h)
    an = float((lam0.cpu().numpy() * v).sum())
    assert abs(fd - an) <= TOL_FD * abs(fd), (fd, an, abs(fd - an) / abs(fd))
    dg.close()
