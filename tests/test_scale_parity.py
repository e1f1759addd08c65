"""Parity at the full size of the vortex configurations (HLLC, MUSCL linear,
Venkatakrishnan, SSP-RK3 at CFL 0.8, global adaptive time step):

* 1024 x 1024 quads, half split (1,572,864 cells): three steps of the exact
  variant against the oracle bit for bit, where index arithmetic or the time
  step's minimum over all cells could differ from the small meshes;
* the same mesh and the all-triangle 1024 x 1024 mesh (2,097,152 cells):
  100 steps of the fast variant (the benchmarked one) and of the exact
  variant against 100 oracle steps.  The bar: the initial residual within
  1e-12 and the state after 100 steps within 1e-9 (max-norm, relative to the
  oracle's maximum); the exact variant bit for bit.

The oracle's runs take a few minutes of one host core each; they run in
spawned worker processes, started once for the module, while the device
marches."""

import multiprocessing as mp
from concurrent.futures import ProcessPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 100
TOL_RESIDUAL = 1e-12
TOL_STATE = 1e-9
SPLITS = ("half", "all")
CELLS = {"half": 1572864, "all": 2097152}


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def oracle_runs(cuda_device):
    from oracle.scale import vortex_run

    pool = ProcessPoolExecutor(max_workers=len(SPLITS), mp_context=mp.get_context("spawn"))
    futures = {split: pool.submit(vortex_run, 1024, split, STEPS) for split in SPLITS}
    yield futures
    pool.shutdown(cancel_futures=True)


def _device_run(split, cuda_device):
    import torch
    from meshcfd_gb300.device import DeviceGeometry, primitive_to_conservative
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, vortex_case, vortex_primitive

    case, _ = vortex_case(1024, split=split)
    g = build_geometry(case.mesh, case)
    s = case.numerics
    s.end_time, s.residual_tolerance = 1.0e30, 1e-300
    U0 = primitive_to_conservative(vortex_primitive(cell_centroids(case.mesh)), s.gamma)
    return DeviceGeometry(g, cuda_device), s, U0, torch.as_tensor(U0, device=cuda_device)


def test_full_size_vortex_steps_match_the_oracle_bit_for_bit(cuda_device, oracle_runs):
    import torch
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import vortex_case
    from meshcfd_gb300.solver import run_explicit
    from oracle.oracle import GeometryHost, Oracle

    dg, s, U0, U = _device_run("half", cuda_device)
    assert dg.n_cells == CELLS["half"]
    s.max_iterations = 3
    case, _ = vortex_case(1024, split="half")
    ref, t_ref = Oracle(build_geometry(case.mesh, case, host=GeometryHost())).solve(U0, s, 3)
    result = run_explicit(dg, s, U, final_residual=False)
    assert result.steps == 3 and abs(result.time - t_ref) <= 1e-12 * t_ref
    np.testing.assert_array_equal(U.cpu().numpy(), ref)
    dg.close()
    torch.cuda.empty_cache()


@pytest.mark.parametrize("split", SPLITS)
def test_full_size_vortex_100_steps_match_the_oracle(cuda_device, oracle_runs, split):
    import torch
    from meshcfd_gb300.device import make_config
    from meshcfd_gb300.solver import run_explicit

    dg, s, U0, U = _device_run(split, cuda_device)
    assert dg.n_cells == CELLS[split]
    s.max_iterations = STEPS
    finals = {}
    for mode in ("fast", "exact"):
        U.copy_(torch.as_tensor(U0, device=cuda_device))
        R = dg.residual(U, make_config(s, mode))
        dg.check_status()
        result = run_explicit(dg, s, U, mode=mode, final_residual=False)
        assert result.steps == STEPS
        finals[mode] = (R.cpu().numpy(), U.cpu().numpy(), result.time)
    dg.close()
    torch.cuda.empty_cache()
    ref = oracle_runs[split].result(timeout=1800)
    assert ref["cells"] == CELLS[split]
    for mode, (R, UN, t) in finals.items():
        assert _rel(R, ref["R0"]) <= TOL_RESIDUAL, (mode, _rel(R, ref["R0"]))
        assert _rel(UN, ref["U"]) <= TOL_STATE, (mode, _rel(UN, ref["U"]))
        assert abs(t - ref["time"]) <= 1e-12 * ref["time"], (mode, t, ref["time"])
    # the exact variant is the reference's operation order: bit for bit
    np.testing.assert_array_equal(finals["exact"][0], ref["R0"])
    np.testing.assert_array_equal(finals["exact"][1], ref["U"])
