"""Batched cases: the concatenated geometry computes exactly what each case
computes alone (CPU: oracle; GPU: kernels, per-case time steps, CUDA graph)."""

import numpy as np
import pytest


def _small_batch():
    from meshcfd_gb300.batch import build_batch, channel_riemann_case

    cases = [channel_riemann_case(c, a, m, 40 + k) for k, (c, a, m) in
             enumerate(((300, 1.0, 0.5), (800, 3.0, 1.7), (150, 2.2, 0.3), (500, 1.5, 1.1)))]
    return cases, build_batch(cases)


def test_batch_residual_equals_per_case_residuals_oracle():
    from oracle.oracle import Oracle

    cases, (geo, layout, P0, geoms) = _small_batch()
    s = cases[0][0].numerics
    big = Oracle(geo)
    U = big.conservative(P0, s.gamma)
    R = big.residual(U, s)
    dt = big.stable_time_steps(big.primitive(U, s.gamma), s)
    for k, g in enumerate(geoms):
        a, b = layout.cell_offsets[k], layout.cell_offsets[k + 1]
        orc = Oracle(g)
        np.testing.assert_array_equal(R[a:b], orc.residual(U[a:b], s))
        np.testing.assert_array_equal(dt[a:b], orc.stable_time_steps(orc.primitive(U[a:b], s.gamma), s))


def test_batch_workload_statistics():
    from meshcfd_gb300.batch import batch_workload

    rng = np.random.default_rng(3)
    cells = np.exp(rng.uniform(np.log(2000), np.log(200000), 256)).astype(int)
    assert 2000 <= cells.min() and cells.max() <= 200000
    assert 5e6 < cells.sum() < 2e7
    cases = batch_workload(n_cases=3, low=2000, high=4000)
    assert all(1500 < len(c.mesh.cells) < 5000 for c, _ in cases)


@pytest.mark.gpu
def test_batch_steps_equal_single_case_steps(cuda_device):
    import torch
    from meshcfd_gb300.batch import BatchStepper
    from meshcfd_gb300.device import DeviceGeometry, make_config
    from meshcfd_gb300.solver import run_explicit
    from oracle.oracle import Oracle

    cases, (geo, layout, P0, geoms) = _small_batch()
    s = cases[0][0].numerics
    U0 = Oracle(geo).conservative(P0, s.gamma)
    dg = DeviceGeometry(geo)
    cfg = make_config(s, "fast")
    R = dg.residual(torch.as_tensor(U0, device=cuda_device), cfg).cpu().numpy()
    stepper = BatchStepper(dg, layout, s, mode="fast")
    U = torch.as_tensor(U0, device=cuda_device)
    for _ in range(5):
        stepper.step(U)
    dg.check_status()
    Ub = U.cpu().numpy()
    # the same steps captured in a CUDA graph
    Ug = torch.as_tensor(U0, device=cuda_device)
    stepper.capture(Ug, 4)          # capture runs one warm-up step eagerly
    stepper.replay()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(Ug.cpu().numpy(), Ub)
    for k, g in enumerate(geoms):
        a, b = layout.cell_offsets[k], layout.cell_offsets[k + 1]
        single = DeviceGeometry(g)
        np.testing.assert_array_equal(R[a:b], single.residual(torch.as_tensor(U0[a:b], device=cuda_device), cfg).cpu().numpy())
        Uk = torch.as_tensor(U0[a:b], device=cuda_device)
        s.max_iterations = 5
        run_explicit(single, s, Uk, mode="fast", final_residual=False)
        np.testing.assert_array_equal(Uk.cpu().numpy(), Ub[a:b])


@pytest.mark.gpu
def test_batched_adjoint_equals_single_case_adjoints(cuda_device):
    """One reverse sweep over the concatenated batch gives every case its own
    wall-force gradient, bit for bit what the case's own adjoint gives (each
    case with its own fixed time step, per-cell in the batch)."""
    import torch
    from meshcfd_gb300.adjoint import WallForceAdjoint
    from meshcfd_gb300.device import DeviceGeometry
    from oracle.oracle import Oracle

    cases, (geo, layout, P0, geoms) = _small_batch()
    s = cases[0][0].numerics
    U0 = Oracle(geo).conservative(P0, s.gamma)
    off = layout.cell_offsets
    dts = []
    for k, g in enumerate(geoms):
        orc = Oracle(g)
        dts.append(0.5 * float(orc.stable_time_steps(orc.primitive(U0[off[k]:off[k + 1]], s.gamma), s).min()))
    dt_cells = torch.as_tensor(np.repeat(dts, np.diff(off)), device=cuda_device)
    steps, every = 9, 4
    d = (0.0, 1.0)  # the channels' walls are horizontal
    adj = WallForceAdjoint(DeviceGeometry(geo), s, dt_cells, direction=d, checkpoint_every=every, mode="fast",
                           case_offsets=off)
    U = torch.as_tensor(U0, device=cuda_device)
    UN = adj.forward(U, steps)
    J_cases = adj.functional_per_case(UN)
    _, dJ = adj.functional(UN)
    lam = adj.backward(dJ).cpu().numpy()
    far = adj.far_acc.cpu().numpy()
    far_start = 0
    for k, g in enumerate(geoms):
        single = WallForceAdjoint(DeviceGeometry(g), s, dts[k], direction=d, checkpoint_every=every, mode="fast")
        Jk, lam_k, far_k = single.gradient(torch.as_tensor(U0[off[k]:off[k + 1]], device=cuda_device), steps)
        assert abs(Jk) > 1e-3 and float(np.abs(lam_k.cpu().numpy()).max()) > 1e-6
        np.testing.assert_array_equal(lam[off[k]:off[k + 1]], lam_k.cpu().numpy())
        nf = len(g.far_field_faces)
        # far-field weights: dt per face owner in the batch, a scalar alone
        # (another rounding order of the same products)
        assert np.abs(far[far_start:far_start + nf] - far_k[:nf]).max() <= 1e-13 * np.abs(far_k[:nf]).max()
        far_start += nf
        assert abs(J_cases[k] - Jk) <= 1e-12 * abs(Jk)
