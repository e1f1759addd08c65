"""GPU implicit Euler against the reference (golden) and the oracle.

Tolerances: the LU-SGS application and the preconditioner are deterministic
(1e-12); the finite-difference operator divides a residual difference by
eps ~ 1.5e-8 |u| / |v|, so last-place differences in the norms that set eps
(deterministic trees here, BLAS in the reference) appear at ~1e-8 relative
(bound 1e-6); GMRES iterates inherit that, and the converged Newton states
agree with the reference-made fixtures within 1e-12 (measured 1.6e-16 to
5e-15).
"""

import ctypes as C

import numpy as np
import pytest

from conftest import load_fixture, solve_settings

pytestmark = pytest.mark.gpu

FIXTURES = ("implicit_channel.npz", "implicit_periodic.npz")


def _prepared(name, cuda_device):
    import torch
    from dataclasses import replace
    from meshcfd_gb300.device import DeviceGeometry, make_config

    data, geom = load_fixture(name)
    s = solve_settings(data)
    dg = DeviceGeometry(geom)
    cfg = make_config(s)
    U = torch.as_tensor(data["U"], device=cuda_device)
    dt = torch.as_tensor(data["dt_cells"], device=cuda_device)
    scales = (C.c_double * 4)(*data["scales"])
    rc = dg.lib.mcfd_implicit_prepare(dg.handle, C.byref(cfg), U.data_ptr(), dt.data_ptr(), 1, scales,
                                      torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    dg.check_status()
    return data, geom, s, dg, U, dt


@pytest.mark.parametrize("name", FIXTURES)
def test_lusgs_apply_matches_reference(cuda_device, name):
    import torch

    data, geom, s, dg, U, dt = _prepared(name, cuda_device)
    v = torch.as_tensor(data["v"], device=cuda_device)
    x = torch.empty_like(v)
    assert dg.lib.mcfd_lusgs_apply(dg.handle, v.data_ptr(), x.data_ptr(), torch.cuda.current_stream().cuda_stream) == 0
    ref = data["lusgs_v"]
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("name", FIXTURES)
def test_fd_operator_matches_reference(cuda_device, name):
    import torch

    data, geom, s, dg, U, dt = _prepared(name, cuda_device)
    v = torch.as_tensor(data["v"], device=cuda_device)
    out = torch.empty_like(v)
    assert dg.lib.mcfd_implicit_matvec(dg.handle, v.data_ptr(), out.data_ptr(),
                                       torch.cuda.current_stream().cuda_stream) == 0
    dg.check_status()
    ref = data["operator_v"]
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("name", FIXTURES)
def test_gmres_solves_to_the_reference_tolerance(cuda_device, name):
    """GMRES(m) with LU-SGS at the case's own tolerance: the GPU solution
    meets SciPy's stopping rule (true residual <= tol |b|) measured with the
    oracle's operator, in about as many iterations as SciPy needs."""
    import torch
    from dataclasses import replace
    from oracle.implicit import ImplicitOracle
    from oracle.oracle import OracleError

    data, geom, s, dg, U, dt = _prepared(name, cuda_device)
    tol = s.gmres_tolerance
    b = torch.as_tensor(data["v"], device=cuda_device)
    x = torch.empty_like(b)
    iters = C.c_int32(0)
    rc = dg.lib.mcfd_gmres(dg.handle, b.data_ptr(), x.data_ptr(), tol, 300, s.gmres_krylov_dimension,
                           C.byref(iters), torch.cuda.current_stream().cuda_stream)
    imp = ImplicitOracle(geom)
    first = replace(s, reconstruction="First order")
    M = imp.preconditioner(data["P0"], first, data["dt_cells"])
    op = imp.operator(data["U"], imp.orc.residual(data["U"], first), data["scales"][None, :], data["dt_cells"], first)
    try:
        ref, used = imp.solve_gmres(op, M, data["v"], tol, 300, s.gmres_krylov_dimension)
    except OracleError:
        # SciPy does not converge on this system within 300 iterations either
        assert rc == 6, rc
        assert iters.value == 300
        return
    assert rc == 0, rc
    got = x.cpu().numpy()
    res = np.linalg.norm(data["v"] - op.matvec(got)) / np.linalg.norm(data["v"])
    assert res <= 1.5 * tol, res
    assert abs(iters.value - used) <= max(3, used // 10), (iters.value, used)


@pytest.mark.parametrize("name", FIXTURES)
def test_implicit_solve_matches_reference(cuda_device, name):
    import torch
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.implicit import run_implicit
    from oracle.oracle import Oracle

    data, geom = load_fixture(name)
    s = solve_settings(data)
    dg = DeviceGeometry(geom)
    U = torch.as_tensor(data["U"], device=cuda_device)
    time, steps, _ = run_implicit(dg, s, U, max_steps=int(data["steps"]))
    P = Oracle(geom).primitive(U.cpu().numpy(), s.gamma)
    ref = data["P_final"]
    assert steps == int(data["steps"])
    err = np.abs(P - ref).max() / np.abs(ref).max()
    print(f"{name}: {steps} implicit steps against the reference, max relative difference {err:.2e}")
    assert err <= 1e-12, err  # measured 1.6e-16 (channel, 4 steps) and 5.0e-15 (periodic, 3 steps)
    assert abs(time - float(data["time"])) <= 1e-9 * float(data["time"])


def test_bump_step_matches_the_reference_made_step(cuda_device):
    """tests/golden/implicit_bump.npz, the reference's own implicit-Euler step
    on a 16x8 bump (nine time-step halvings before its Newton solve
    converges): the device step takes the same halvings to the same state."""
    import torch
    from conftest import ROOT
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.implicit import ImplicitEuler
    from meshcfd_gb300.meshes import bump_case

    data = np.load(ROOT / "tests" / "golden" / "implicit_bump.npz")
    case, _ = bump_case(16, 8)
    dg = DeviceGeometry(build_geometry(case.mesh, case))
    stepper = ImplicitEuler(dg, case.numerics)
    U = torch.as_tensor(data["U"], device=cuda_device)
    out, used = stepper.step(U, torch.as_tensor(data["dt"], device=cuda_device))
    np.testing.assert_array_equal(used.cpu().numpy(), data["used"])
    err = np.abs(out.cpu().numpy() - data["U_next"]).max() / np.abs(data["U_next"]).max()
    print(f"bump 16x8, the reference's step: max relative difference {err:.2e}")
    assert err <= 1e-12, err


def test_implicit_conserves_periodic_state(cuda_device):
    """The reference's own implicit test idea (tests/test_solver.py:735-783):
    on a periodic mesh an implicit step conserves the integrated state."""
    import torch
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.implicit import run_implicit
    from meshcfd_gb300.meshes import periodic_case, smooth_primitive
    from oracle.oracle import Oracle

    case = periodic_case(12, 9, split="half", jitter=0.2, seed=5)
    s = case.numerics
    s.flux, s.reconstruction, s.time_integration = "Rusanov", "MUSCL linear", "Implicit Euler"
    s.cfl, s.end_time, s.max_iterations = 100.0, 1e30, 2
    g = build_geometry(case.mesh, case)
    orc = Oracle(g)
    U0 = orc.conservative(smooth_primitive(len(g.areas), seed=3), s.gamma)
    dg = DeviceGeometry(g)
    U = torch.as_tensor(U0, device=cuda_device)
    run_implicit(dg, s, U)
    before = (U0 * g.areas[:, None]).sum(axis=0)
    after = (U.cpu().numpy() * g.areas[:, None]).sum(axis=0)
    np.testing.assert_allclose(after, before, rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("nx,ny,n_steps", ((32, 16, 3), (128, 64, 1)))
def test_bump_channel_implicit_steps_match_the_oracle(cuda_device, nx, ny, n_steps):
    """The bump-channel recipe (circular-arc bump, rows stretched toward the
    wall, slip wall, far field and pressure outlet; Roe, MUSCL linear with
    Barth-Jespersen, implicit Euler with local steps at CFL 200, GMRES(30) to
    1e-3 with LU-SGS) on a 32x16 mesh (three implicit steps) and a 128x64
    mesh (one step: ten time-step halvings, ~80 Newton and ~2,000 GMRES
    iterations, 191 sweep levels) on the device against the oracle's
    restatement with SciPy's GMRES."""
    import torch
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.implicit import run_implicit
    from meshcfd_gb300.meshes import bump_case
    from oracle.implicit import ImplicitOracle
    from oracle.oracle import Oracle

    case, P = bump_case(nx, ny)
    s = case.numerics
    g = build_geometry(case.mesh, case)
    assert len(g.wall_faces) and len(g.far_field_faces) and len(g.pressure_outlet_faces)
    orc, imp = Oracle(g), ImplicitOracle(g)
    U0 = orc.conservative(P, s.gamma)
    U_ref = U0.copy()
    for _ in range(n_steps):
        dt = orc.stable_time_steps(orc.primitive(U_ref, s.gamma), s)
        U_ref, _ = imp.step(U_ref, dt, s)
    dg = DeviceGeometry(g)
    U = torch.as_tensor(U0, device=cuda_device)
    _, steps, _ = run_implicit(dg, s, U, max_steps=n_steps)
    assert steps == n_steps
    err = np.abs(U.cpu().numpy() - U_ref).max() / np.abs(U_ref).max()
    print(f"bump {nx}x{ny}, {n_steps} implicit steps: max relative difference {err:.2e}")
    assert err <= 1e-12, err  # measured 1.6e-16 on 32x16: the GMRES iterates track SciPy's


def _prepare_on(g, s, P, cuda_device):
    """An implicit operator prepared on geometry g at primitive state P with
    the recipe's local time steps and the Newton scales of the state."""
    import torch
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from oracle.implicit import ImplicitOracle
    from oracle.oracle import Oracle

    orc = Oracle(g)
    U0 = orc.conservative(P, s.gamma)
    dt = orc.stable_time_steps(P, s)
    scales = ImplicitOracle.scales(U0, P, s.gamma)[0]
    dg = DeviceGeometry(g)
    cfg = make_config(s)
    U = torch.as_tensor(U0, device=cuda_device)
    dtd = torch.as_tensor(dt, device=cuda_device)
    assert dg.lib.mcfd_implicit_prepare(dg.handle, C.byref(cfg), U.data_ptr(), dtd.data_ptr(), 1,
                                        (C.c_double * 4)(*scales), torch.cuda.current_stream().cuda_stream) == 0
    dg.check_status()
    return dg, U0, dt, scales


def _permuted_periodic(n, seed):
    """A periodic mesh whose cell and face ids are randomly permuted: its
    LU-SGS levels are few and wide and rows depend on far-away positions."""
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import periodic_case, permute_mesh

    case = periodic_case(n, n, split="half", jitter=0.2, seed=5)
    rng = np.random.default_rng(seed)
    case.mesh = permute_mesh(case.mesh, rng.permutation(len(case.mesh.cells)), rng.permutation(len(case.mesh.faces)))
    s = case.numerics
    s.flux, s.reconstruction, s.time_integration, s.cfl = "Roe", "MUSCL linear", "Implicit Euler", 50.0
    s.time_step_mode = "Local (steady)"
    return case, build_geometry(case.mesh, case)


@pytest.mark.parametrize("mesh", ("bump", "permuted", "bump512", "permuted192"))
def test_lusgs_schedules_agree_and_match_spsolve(cuda_device, mesh):
    """Every launch schedule of the level-scheduled sweeps (one block with a
    barrier per level, one block whose rows wait only for the rows they read,
    or a cluster of 8 or 16, stepping through narrow levels with their
    shared-memory rings, either sharing every solution or each block owning
    a band of cells; grid launches per level; and mixtures) gives the
    same bits, and matches the reference's two spsolve_triangular calls
    (within 1e-12)."""
    import torch
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import bump_case, smooth_primitive
    from oracle.implicit import ImplicitOracle
    from dataclasses import replace

    if mesh.startswith("bump"):
        case, P = bump_case(*((512, 256) if mesh == "bump512" else (96, 48)))
        P = P * (1.0 + 0.05 * np.random.default_rng(4).standard_normal(P.shape))
        s = case.numerics
        g = build_geometry(case.mesh, case)
    else:
        # randomly numbered cells: rows read solutions far back in sweep
        # order (beyond the dataflow sweep's shared-memory window)
        case, g = _permuted_periodic(192 if mesh == "permuted192" else 64, 7)
        s = case.numerics
        P = smooth_primitive(len(g.areas), seed=3)
    dg, U0, dt, _ = _prepare_on(g, s, P, cuda_device)
    v = torch.as_tensor(np.random.default_rng(2).standard_normal(U0.shape), device=cuda_device)
    stream = torch.cuda.current_stream().cuda_stream
    outs = []
    for wide, engine, chunk in ((0, 1, 0), (0, 2, 0), (0, 3, 0), (0, 4, 0), (0, 5, 0), (7, 5, 0), (0, 6, 0), (0, 6, 3), (7, 6, 0),
                                (1 << 30, 6, 0), (0, 2, 1), (0, 4, 8), (0, 2, 17),
                                (0, 8, 0), (0, 16, 0), (1, 8, 0), (7, 1, 0), (7, 2, 0), (7, 3, 5), (7, 8, 0),
                                (1 << 30, 1, 0), (1 << 30, 2, 0), (1 << 30, 3, 0), (1 << 30, 16, 0),
                                (0, 7, 0), (0, 9, 0), (7, 7, 0), (1, 9, 0), (1 << 30, 7, 0), (1 << 30, 9, 0)):
        assert dg.lib.mcfd_implicit_set_chunk(dg.handle, chunk) == 0
        rc = dg.lib.mcfd_implicit_set_sweep(dg.handle, wide, engine)
        if engine > 2 and rc == 3:
            continue  # the device cannot run this cluster size
        assert rc == 0
        x = torch.empty_like(v)
        assert dg.lib.mcfd_lusgs_apply(dg.handle, v.data_ptr(), x.data_ptr(), stream) == 0
        outs.append(x.cpu().numpy())
    dg.check_status()
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])
    M = ImplicitOracle(g).preconditioner(P, replace(s, reconstruction="First order"), dt)
    ref = M.matvec(v.cpu().numpy().ravel()).reshape(U0.shape)
    assert np.abs(outs[0] - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("exact_jacobian", (0, 1))
def test_gmres_captured_inner_loop_equals_host_stepping(cuda_device, exact_jacobian):
    """The restart cycle as a CUDA graph with a device-set loop condition
    against the same Arnoldi steps driven from the host one at a time (the
    path taken while profiling events are recorded): equal iteration counts
    and solutions bit for bit, twice in a row (graph reuse), with both
    Jacobians."""
    import torch
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import bump_case

    case, P = bump_case(48, 24)
    P = P * (1.0 + 0.05 * np.random.default_rng(5).standard_normal(P.shape))
    s = case.numerics
    g = build_geometry(case.mesh, case)
    dg, U0, dt, _ = _prepare_on(g, s, P, cuda_device)
    assert dg.lib.mcfd_implicit_set_jacobian(dg.handle, exact_jacobian) == 0
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(9)
    for _ in range(2):
        b = torch.as_tensor(rng.standard_normal(U0.shape), device=cuda_device)
        results = []
        for profiling in (0, 1):
            dg.lib.mcfd_profile_enable(dg.handle, profiling)
            x = torch.empty_like(b)
            it = C.c_int32(0)
            rc = dg.lib.mcfd_gmres(dg.handle, b.data_ptr(), x.data_ptr(), 1e-3, 120, 30, C.byref(it), stream)
            results.append((rc, it.value, x.cpu().numpy()))
        dg.lib.mcfd_profile_enable(dg.handle, 0)
        dg.check_status()
        (rc0, it0, x0), (rc1, it1, x1) = results
        assert rc0 == rc1 and rc0 in (0, 6) and it0 == it1 and it0 > 30  # more than one restart cycle
        np.testing.assert_array_equal(x0, x1)
