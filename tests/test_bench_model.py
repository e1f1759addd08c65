"""The algorithmic byte model behind the bench's roofline figure (the
reference 3-pass model: every array the reference algorithm produces or
consumes moves once per pass) on the two vortex meshes."""

import numpy as np


def _step_bytes_per_cell(g):
    import bench

    m, n = bench.model_bytes(g)
    C = n["C"]
    per_cell = {k: v / C for k, v in m.items()}
    # RK3: three stages of reconstruct + flux + gather, the first stage
    # reading U^0 once, and one time-step pass
    step = 3 * (m["reconstruct"] + m["flux"] + m["gather"]) - 32 * C + m["time_step"]
    return per_cell, step / C, n


def test_all_triangle_periodic_mesh_moves_2036_bytes_per_cell_update():
    """F = 1.5 C, E = L = 3 C: 236 + 272 + 152 B per cell per stage and
    88 B for the time step, 2,036 B per RK3 cell-update."""
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import vortex_case

    case, _ = vortex_case(16, split="all")
    per_cell, step, n = _step_bytes_per_cell(build_geometry(case.mesh, case))
    assert n["F"] * 2 == 3 * n["C"] and n["E"] == 3 * n["C"] and n["L"] == 3 * n["C"]
    assert (per_cell["reconstruct"], per_cell["flux"], per_cell["gather"], per_cell["time_step"]) == (236, 272, 152, 88)
    assert step == 2036


def test_mixed_vortex_mesh_moves_about_2142_bytes_per_cell_update():
    """Half the quads split (F / C = 5/3): 2,141.3 B per RK3 cell-update."""
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import vortex_case

    case, _ = vortex_case(32, split="half")
    _, step, n = _step_bytes_per_cell(build_geometry(case.mesh, case))
    assert np.isclose(n["F"] / n["C"], 5.0 / 3.0)
    assert abs(step - 2142) <= 1.0


def test_reference_arm_sample_fits_its_cpu_budget():
    """The reference arm times the full mesh when its steps fit ~3 min of
    one core, else the same recipe at 512^2 or 256^2 quads."""
    import bench

    assert bench.reference_sample("vortex1024", 100, 3) == 1024
    assert bench.reference_sample("vortex1024", 300, 3) == 512
    assert bench.reference_sample("vortex1024", 1000, 3) == 256
    case, settings, g, P0 = bench._sample_case("vortex1024", 16)
    assert len(g.areas) == 16 * 16 * 3 // 2 == len(P0)
    assert settings.flux == "HLLC" and settings.limiter == "Venkatakrishnan"
