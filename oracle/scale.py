"""ORACLE — test infrastructure only: full-size oracle runs for parity tests.

The worker functions here run in spawned processes (no CUDA in them), so a
GPU test can march the device path while the oracle's single-threaded runs
of the same recipes proceed on other host cores.  They build the geometry
with the oracle's own restatement of the reference's geometry loops.
"""

from __future__ import annotations


def vortex_run(n: int, split: str, steps: int) -> dict:
    """The isentropic-vortex recipe (HLLC, MUSCL linear, Venkatakrishnan,
    SSP-RK3 at CFL 0.8, global adaptive time step) at ``n`` x ``n`` quads:
    the residual of the initial state and the state after ``steps`` steps of
    the reference's explicit loop (solver.py:437-806), with the time reached."""
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, vortex_case, vortex_primitive
    from oracle.oracle import GeometryHost, Oracle

    case, _ = vortex_case(n, split=split)
    g = build_geometry(case.mesh, case, host=GeometryHost())
    s = case.numerics
    orc = Oracle(g)
    U0 = orc.conservative(vortex_primitive(cell_centroids(case.mesh)), s.gamma)
    R0 = orc.residual(U0, s)
    U, t = orc.solve(U0, s, steps)
    return {"cells": len(g.areas), "R0": R0, "U": U, "time": t}
