"""The drop-in boundary (`meshcfd_gb300.dropin`): the reference solver
module's functions replaced in place, as the reference's own tests replace
them with monkeypatch (tests/test_solver.py:1300-1306).  A stand-in module
with the reference's function names plays `meshcfd.core.solver`."""

import types

import numpy as np
import pytest
import torch

NAMES = ("_residual", "_stable_time_steps", "_stable_time_step", "_explicit_rk4_step", "_implicit_euler_step")


class _SolverError(ValueError):
    pass


def _module():
    def original(*args, **kwargs):
        raise AssertionError("the reference function ran instead of the GPU one")

    return types.SimpleNamespace(SolverError=_SolverError, **{name: original for name in NAMES})


def _vortex():
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, vortex_case, vortex_primitive

    case, _ = vortex_case(12, split="half")
    return case, build_geometry(case.mesh, case), vortex_primitive(cell_centroids(case.mesh))


def test_install_patches_the_reference_functions_and_uninstall_restores_them():
    from meshcfd_gb300 import dropin

    module = _module()
    before = {name: getattr(module, name) for name in NAMES}
    originals = dropin.install(module)
    assert originals == before
    for name in NAMES:
        patched = getattr(module, name)
        assert patched is not before[name] and patched.__name__ == name
    dropin.uninstall(module, originals)
    assert {name: getattr(module, name) for name in NAMES} == before


def test_turbulence_states_are_refused_before_any_device_work():
    from meshcfd_gb300 import dropin

    case, g, P = _vortex()
    module = _module()
    dropin.install(module)
    U = np.ones((len(P), 4))
    with pytest.raises(NotImplementedError, match="SST"):
        module._residual(U, g, case.numerics, np.ones((len(P), 2)))
    with pytest.raises(NotImplementedError, match="SST"):
        module._stable_time_steps(P, g, case.numerics, np.ones((len(P), 2)))
    with pytest.raises(NotImplementedError, match="SST"):
        module._explicit_rk4_step(np.ones((len(P), 6)), 0.1, g, case.numerics)
    with pytest.raises(NotImplementedError, match="SST"):
        module._implicit_euler_step(np.ones((len(P), 6)), 0.1, g, case.numerics)


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a CUDA device")
def test_without_a_device_the_patched_functions_raise_instead_of_falling_back():
    from meshcfd_gb300 import dropin

    case, g, P = _vortex()
    module = _module()
    dropin.install(module)
    with pytest.raises(RuntimeError):
        module._residual(np.ones((len(P), 4)), g, case.numerics)


@pytest.mark.gpu
def test_patched_functions_match_the_oracle(cuda_device):
    """Residual, per-cell and global stable time steps and the SSPRK(5,4)
    step through the patched module functions (NumPy in, NumPy out) on the
    periodic vortex: bit-exact against the oracle."""
    from meshcfd_gb300 import dropin
    from oracle.oracle import Oracle

    case, g, P = _vortex()
    s = case.numerics
    s.flux, s.reconstruction, s.limiter, s.time_integration = "HLLC", "MUSCL linear", "Venkatakrishnan", "Explicit RK4"
    orc = Oracle(g)
    U = orc.conservative(P, s.gamma)
    module = _module()
    originals = dropin.install(module)
    try:
        np.testing.assert_array_equal(module._residual(U, g, s), orc.residual(U, s))
        dt_ref = orc.stable_time_steps(P, s)
        np.testing.assert_array_equal(module._stable_time_steps(P, g, s), dt_ref)
        assert module._stable_time_step(P, g, s) == float(np.min(dt_ref))
        dt = float(np.min(dt_ref))
        np.testing.assert_array_equal(module._explicit_rk4_step(U, dt, g, s), orc.explicit_step(U, s, dt))
    finally:
        dropin.uninstall(module, originals)


@pytest.mark.gpu
def test_patched_implicit_step_matches_the_oracle(cuda_device):
    """One implicit-Euler step of the bump-channel recipe (32 x 16) through
    the patched `_implicit_euler_step`, against the oracle's restatement with
    SciPy's GMRES."""
    from meshcfd_gb300 import dropin
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import bump_case
    from oracle.implicit import ImplicitOracle
    from oracle.oracle import Oracle

    case, P = bump_case(32, 16)
    s = case.numerics
    g = build_geometry(case.mesh, case)
    orc = Oracle(g)
    U = orc.conservative(P, s.gamma)
    dt = orc.stable_time_steps(P, s)
    ref, used_ref = ImplicitOracle(g).step(U, dt, s)
    module = _module()
    originals = dropin.install(module)
    try:
        got, used = module._implicit_euler_step(U, dt, g, s)
    finally:
        dropin.uninstall(module, originals)
    np.testing.assert_array_equal(used, used_ref)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def _checking_module(check):
    """A stand-in whose ``solve_case`` runs ``check`` (the reference's
    prologue) and then builds the geometry, as solver.py:193-379 does."""
    calls = []

    def build(mesh, case):
        calls.append("build")
        return "geometry"

    def solve_case(case, start_time=0.0, step_offset=0, solution_interval=1):
        check(case, start_time, step_offset, solution_interval)
        module._build_geometry(case.mesh, case)
        raise AssertionError("the reference loop ran past its geometry build")

    module = types.SimpleNamespace(SolverError=_SolverError, _build_geometry=build, solve_case=solve_case)
    return module, build, calls


def test_the_hbm_loop_runs_the_reference_checks_and_restores_the_builder():
    """dropin.solve_case's prologue: the reference's own checks raise its
    SolverError with its message; a case that passes them stops at the
    geometry build, which does not run; the module's builder is the
    reference's again either way."""
    from meshcfd_gb300 import dropin

    def check(case, start_time, step_offset, solution_interval):
        if solution_interval <= 0:
            raise _SolverError("Solution output interval must be a positive integer.")

    module, build, calls = _checking_module(check)
    case = types.SimpleNamespace(mesh="mesh")
    with pytest.raises(_SolverError, match="Solution output interval"):
        dropin._reference_checks(module, case, 0.0, 0, 0)
    assert module._build_geometry is build and calls == []
    assert dropin._reference_checks(module, case, 0.0, 0, 1) is None
    assert module._build_geometry is build and calls == []


def test_the_hbm_loop_refuses_a_reference_that_skips_its_geometry_build():
    from meshcfd_gb300 import dropin

    module = types.SimpleNamespace(SolverError=_SolverError, _build_geometry=lambda mesh, case: None,
                                   solve_case=lambda case, **kw: None)
    before = module._build_geometry
    with pytest.raises(RuntimeError, match="returned before its geometry build"):
        dropin._reference_checks(module, types.SimpleNamespace(mesh="mesh"), 0.0, 0, 1)
    assert module._build_geometry is before
