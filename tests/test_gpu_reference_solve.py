"""The reference's own ``solve_case`` (meshcfd.core.solver, solver.py:179-1001)
running on the GPU path: the drop-in replaces the module's hot-path
functions in place, as the reference's tests do with monkeypatch
(tests/test_solver.py:1300-1306), and the reference's unmodified loop, with
its stage combinations, time-step logic, progress residuals and primitive
checks, calls them.  Checked against the oracle at the configurations'
128^2 size, and against the reference's own CPU ``solve_case`` on small
meshes.

Needs the reference package (an offline install of it under baseline/_ref,
or a checkout named by MESHCFD_REFERENCE); Numba is absent, so its compiled
kernels run as plain Python behind an identity ``numba.njit``."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

shim = pytest.importorskip("reference_shim")
if not shim.available():
    pytest.skip("the reference package is not installed", allow_module_level=True)

TOL = 1e-12  # per state after the run, relative to the largest value (far-field pow() last places)


@pytest.fixture(scope="module")
def ref():
    return shim.import_reference()


def _recipe(name, n, integrator, steps):
    from meshcfd_gb300.meshes import cell_centroids, riemann_case, vortex_case, vortex_primitive

    if name == "riemann":
        case, P = riemann_case(n)
        if integrator != "Explicit Euler":
            case.numerics.flux, case.numerics.reconstruction = "HLLC", "MUSCL linear"
            case.numerics.limiter, case.numerics.cfl = "Barth-Jespersen", 0.5
    else:
        case, _ = vortex_case(n, split="half")
        P = vortex_primitive(cell_centroids(case.mesh))
    case.numerics.time_integration = integrator
    case.numerics.max_iterations = steps
    return case, P


def _solve(ref, case, P, gpu):
    from meshcfd_gb300 import dropin

    rcase = shim.reference_case(case, ref)
    init = tuple(ref.model.InitialState(*map(float, row)) for row in P)
    progress = []
    originals = dropin.install(ref.solver) if gpu else None
    try:
        result = ref.solver.solve_case(rcase, initial_states=init, progress_callback=progress.append)
    finally:
        if gpu:
            dropin.uninstall(ref.solver, originals)
    states = np.array([(s.density, s.velocity_x, s.velocity_y, s.pressure) for s in result.states])
    return states, result, progress


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("name,integrator,steps", (
    ("riemann", "Explicit Euler", 100),   # the first configuration as stated: Rusanov, first order, CFL 0.5
    ("riemann", "Explicit RK3", 20),
    ("riemann", "Explicit RK4", 20),
    ("vortex", "Explicit RK3", 20),
    ("vortex", "Explicit RK4", 20),
))
def test_reference_solve_case_on_the_gpu_matches_the_oracle(cuda_device, ref, name, integrator, steps):
    from meshcfd_gb300.geometry import build_geometry
    from oracle.oracle import Oracle

    case, P = _recipe(name, 128, integrator, steps)
    states, result, progress = _solve(ref, case, P, gpu=True)
    assert result.steps == steps and not result.completed
    assert progress and progress[-1].step == steps and all(np.all(np.isfinite(p.residuals)) for p in progress)
    orc = Oracle(build_geometry(case.mesh, case))
    U, t = orc.solve(orc.conservative(P, case.numerics.gamma), case.numerics, steps)
    P_ref = orc.primitive(U, case.numerics.gamma)
    assert abs(result.time - t) <= 1e-12 * t
    assert _rel(states, P_ref) <= TOL, _rel(states, P_ref)
    if name == "vortex":  # periodic: no far-field pow(), the reference's operation order bit for bit
        np.testing.assert_array_equal(states, P_ref)


@pytest.mark.parametrize("name,n,integrator", (("riemann", 8, "Explicit RK3"), ("vortex", 8, "Explicit RK4")))
def test_reference_solve_case_gpu_against_its_own_cpu_run(cuda_device, ref, name, n, integrator):
    """The same ``solve_case`` call twice: unpatched (the reference's own CPU
    path, kernels as plain Python) and patched (the GPU path)."""
    case, P = _recipe(name, n, integrator, 5)
    cpu, r_cpu, p_cpu = _solve(ref, case, P, gpu=False)
    gpu, r_gpu, p_gpu = _solve(ref, case, P, gpu=True)
    assert r_cpu.steps == r_gpu.steps == 5
    assert abs(r_cpu.time - r_gpu.time) <= 1e-12 * r_cpu.time
    assert _rel(gpu, cpu) <= TOL, _rel(gpu, cpu)
    assert abs(r_gpu.residual - r_cpu.residual) <= 1e-10 * abs(r_cpu.residual)
    for a, b in zip(p_cpu, p_gpu):
        assert a.step == b.step
        np.testing.assert_allclose(b.residuals, a.residuals, rtol=1e-10)


def _hbm(ref, case, P, **kw):
    """The HBM-resident loop (``dropin.solve_case``) on the reference's case."""
    from meshcfd_gb300 import dropin

    rcase = shim.reference_case(case, ref)
    init = tuple(ref.model.InitialState(*map(float, row)) for row in P)
    progress = []
    result = dropin.solve_case(ref.solver, rcase, initial_states=init, progress_callback=progress.append, **kw)
    states = np.array([(s.density, s.velocity_x, s.velocity_y, s.pressure) for s in result.states])
    return states, result, progress


@pytest.mark.parametrize("name,integrator,mode", (
    ("riemann", "Explicit RK3", "Global adaptive"),
    ("vortex", "Explicit RK4", "Global adaptive"),
    ("riemann", "Explicit Euler", "Global fixed"),
    ("vortex", "Explicit RK2", "Local (steady)"),
))
def test_hbm_loop_against_the_reference_cpu_run(cuda_device, ref, name, integrator, mode):
    """``dropin.solve_case`` (each step's time steps computed by the step
    before, the progress residual the first stage's) against the reference's
    own CPU ``solve_case``: the same states, times, progress reports (the
    RMS of the residual at the start of each step, solver.py:466, 943-950;
    after the step in local steady mode, solver.py:885-903) and final
    residual."""
    case, P = _recipe(name, 8, integrator, 6)
    s = case.numerics
    s.time_step_mode = mode
    if mode == "Global fixed":
        s.fixed_time_step = 2e-3
    s.convergence_history_interval = 2
    cpu, r_cpu, p_cpu = _solve(ref, case, P, gpu=False)
    gpu, r_gpu, p_gpu = _hbm(ref, case, P)
    assert r_cpu.steps == r_gpu.steps == 6 and r_cpu.completed == r_gpu.completed
    assert abs(r_cpu.time - r_gpu.time) <= 1e-12 * r_cpu.time
    assert _rel(gpu, cpu) <= TOL, _rel(gpu, cpu)
    assert abs(r_gpu.residual - r_cpu.residual) <= 1e-10 * abs(r_cpu.residual)
    assert [p.step for p in p_gpu] == [p.step for p in p_cpu] == [2, 4, 6]
    for a, b in zip(p_cpu, p_gpu):
        assert abs(a.time - b.time) <= 1e-12 * a.time and abs(a.time_step - b.time_step) <= 1e-12 * a.time_step
        np.testing.assert_allclose(b.residuals, a.residuals, rtol=1e-10)


@pytest.mark.parametrize("integrator,factor,step", (("Explicit Euler", 4.0, 32), ("Explicit RK3", 6.0, 2)))
def test_hbm_loop_fails_where_the_reference_fails(cuda_device, ref, integrator, factor, step):
    """A fixed time step several times the stable one on the periodic vortex
    (bit-exact on both paths): the state turns non-physical within the step
    the reference names, and both raise its message."""
    case, P = _recipe("vortex", 8, integrator, 200)
    s = case.numerics
    rcase = shim.reference_case(case, ref)
    geometry = ref.solver._build_geometry(rcase.mesh, rcase)
    dt0 = ref.solver._stable_time_step(P, geometry, rcase.numerics, None)
    s.time_step_mode, s.fixed_time_step, s.end_time = "Global fixed", factor * dt0 / s.cfl, 100.0
    message = (f"Solver failed at step {step}: "
               "Euler state has non-finite or non-positive density or pressure.")
    with pytest.raises(ref.solver.SolverError) as cpu_error:
        _solve(ref, case, P, gpu=False)
    assert str(cpu_error.value) == message
    with pytest.raises(ref.solver.SolverError) as gpu_error:
        _hbm(ref, case, P)
    assert str(gpu_error.value) == message


def test_hbm_loop_runs_the_reference_checks(cuda_device, ref):
    """The case and settings checks are the reference's own."""
    case, P = _recipe("vortex", 8, "Explicit RK3", 3)
    case.numerics.cfl = 1.5
    with pytest.raises(ref.solver.SolverError, match=r"Explicit RK3 requires a CFL number in \(0, 1\]"):
        _hbm(ref, case, P)
    case.numerics.cfl = 0.5
    with pytest.raises(ref.solver.SolverError, match="Solution output interval must be a positive integer"):
        _hbm(ref, case, P, solution_interval=0)
    assert ref.solver._build_geometry.__name__ == "_build_geometry"
