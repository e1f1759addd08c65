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
