"""Many independent cases in one device geometry.

Cases are concatenated with offset tables (cells, faces, interior faces,
limiter slots): a batch is a mesh of disconnected components, so every kernel
covers all cases in one launch, and every cell's gathers keep their own case's
entries in the same order — batched results are bit-identical to solving each
case alone.  Each case keeps its own global time step: per-cell stable steps,
a segmented minimum per case (`mcfd_batch_time_steps`), broadcast back to the
cells, then the explicit step with per-cell steps.  A whole step is a fixed
sequence of launches with no host synchronisation, so it is captured once in
a CUDA graph and replayed.
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from .device import DeviceGeometry, TIME_SCHEME_CODES, _stream_ptr, make_config
from .geometry import Geometry, build_geometry
from .meshes import box_mesh, cell_centroids
from .model import Case

# ------------------------------------------------------------------ workload


def channel_riemann_case(cells: int, aspect: float, mach: float, seed: int):
    """Jittered triangulated rectangle [0, aspect] x [0, 1] of about ``cells``
    triangles: slip walls top and bottom, far field left and right at the
    inflow state (rho = 1, p = 1, Mach ``mach`` along x); the initial state is
    that free stream with a Riemann-type step (rho and p x 1.5) in the first
    quarter of the channel."""
    ny = max(2, int(round(math.sqrt(cells / (2.0 * aspect)))))
    nx = max(2, int(round(cells / (2.0 * ny))))
    mesh = box_mesh(nx, ny, aspect, 1.0, split="all", jitter=0.2, seed=seed)
    case = Case(name=f"channel{seed}", mesh=mesh)
    gamma = case.numerics.gamma
    u = mach * math.sqrt(gamma)
    for c in case.boundary_conditions:
        if c.patch_name in ("bottom", "top"):
            c.kind = "Wall"
            c.mechanical_condition = "Slip"
        else:
            c.kind = "Far Field"
            c.values = {"density": 1.0, "velocity_x": u, "velocity_y": 0.0, "pressure": 1.0}
    num = case.numerics
    num.flux, num.reconstruction, num.limiter = "HLLC", "MUSCL linear", "Venkatakrishnan"
    num.time_integration, num.cfl = "Explicit RK3", 0.8
    num.end_time, num.residual_tolerance = 1.0e30, 1e-300
    x = cell_centroids(mesh)[:, 0]
    P = np.tile((1.0, u, 0.0, 1.0), (len(x), 1))
    P[x < 0.25 * aspect, 0] *= 1.5
    P[x < 0.25 * aspect, 3] *= 1.5
    return case, P


def batch_workload(n_cases=256, low=2000, high=200000, seed=3):
    """The seeded batch: cell counts log-uniform in [low, high], aspect ratio
    uniform in [1, 4], inflow Mach uniform in [0.3, 2.0]."""
    rng = np.random.default_rng(seed)
    cells = np.exp(rng.uniform(np.log(low), np.log(high), n_cases)).astype(int)
    aspect = rng.uniform(1.0, 4.0, n_cases)
    mach = rng.uniform(0.3, 2.0, n_cases)
    return [channel_riemann_case(int(c), float(a), float(m), seed * 100000 + k)
            for k, (c, a, m) in enumerate(zip(cells, aspect, mach))]


# ------------------------------------------------------------- concatenation


@dataclass
class BatchLayout:
    cell_offsets: np.ndarray  # [n_cases + 1]
    face_offsets: np.ndarray
    n_cases: int


def concatenate(geometries) -> tuple[Geometry, BatchLayout]:
    """One geometry whose components are the given cases (index arrays
    shifted by the offset tables; boundary groups concatenated case by case,
    which keeps every cell's accumulation order)."""
    cells = np.cumsum([0] + [len(g.areas) for g in geometries])
    faces = np.cumsum([0] + [len(g.face_lengths) for g in geometries])
    interior = np.cumsum([0] + [len(g.interior_faces) for g in geometries])

    def cat(name, shift=None, width=None):
        parts = []
        for k, g in enumerate(geometries):
            a = np.asarray(getattr(g, name))
            if shift == "cell":
                a = a + cells[k]
            elif shift == "face":
                a = a + faces[k]
            parts.append(a)
        out = np.concatenate(parts) if parts else np.empty(0)
        return out.reshape(-1, width) if width else out

    def cat_cells_or_neg(name):
        parts = []
        for k, g in enumerate(geometries):
            a = np.asarray(getattr(g, name))
            parts.append(np.where(a >= 0, a + cells[k], a))
        return np.concatenate(parts)

    def shift_patches(name):
        # boundary patches keep their order case by case, faces shifted
        from dataclasses import replace

        return tuple(replace(b, faces=np.asarray(b.faces, dtype=np.int64) + faces[k])
                     for k, g in enumerate(geometries) for b in getattr(g, name, ()))

    # limiter entries: owner side of every face, then neighbour side of
    # interior faces — over the whole batch (slot ids are positions)
    lim_cells = np.concatenate(
        [np.asarray(g.limiter_cells[: len(g.face_lengths)]) + cells[k] for k, g in enumerate(geometries)]
        + [np.asarray(g.limiter_cells[len(g.face_lengths):]) + cells[k] for k, g in enumerate(geometries)])
    lim_dx = np.concatenate([np.asarray(g.limiter_dx[: len(g.face_lengths)]) for g in geometries]
                            + [np.asarray(g.limiter_dx[len(g.face_lengths):]) for g in geometries])
    lim_dy = np.concatenate([np.asarray(g.limiter_dy[: len(g.face_lengths)]) for g in geometries]
                            + [np.asarray(g.limiter_dy[len(g.face_lengths):]) for g in geometries])
    geo = Geometry(
        centers=cat("centers", width=2), areas=cat("areas"), inverse_areas=cat("inverse_areas"),
        face_centers=cat("face_centers", width=2), face_normals=cat("face_normals", width=2),
        face_lengths=cat("face_lengths"), wall_velocities=cat("wall_velocities", width=2),
        owners=cat("owners", "cell"), neighbours=cat_cells_or_neg("neighbours"), patch_ids=cat("patch_ids"),
        patch_kinds={}, interior_faces=cat("interior_faces", "face"), interior_owners=cat("interior_owners", "cell"),
        interior_neighbours=cat("interior_neighbours", "cell"), interior_normals=cat("interior_normals", width=2),
        interior_lengths=cat("interior_lengths"), interior_owner_offsets=cat("interior_owner_offsets", width=2),
        interior_neighbour_offsets=cat("interior_neighbour_offsets", width=2),
        wall_faces=cat("wall_faces", "face"), symmetry_faces=cat("symmetry_faces", "face"),
        periodic_faces_a=cat("periodic_faces_a", "face"), periodic_faces_b=cat("periodic_faces_b", "face"),
        velocity_inlet_faces=cat("velocity_inlet_faces", "face"),
        velocity_inlet_states=cat("velocity_inlet_states", width=4),
        pressure_outlet_faces=cat("pressure_outlet_faces", "face"),
        pressure_outlet_pressures=cat("pressure_outlet_pressures"),
        far_field_faces=cat("far_field_faces", "face"), far_field_states=cat("far_field_states", width=4),
        pressure_inlets=shift_patches("pressure_inlets"), mass_flow_inlets=shift_patches("mass_flow_inlets"),
        mass_flow_outlets=shift_patches("mass_flow_outlets"),
        gradient_sources=cat("gradient_sources", "cell"), gradient_neighbours=cat("gradient_neighbours", "cell"),
        gradient_dx=cat("gradient_dx"), gradient_dy=cat("gradient_dy"),
        gradient_coefficients_x=cat("gradient_coefficients_x"), gradient_coefficients_y=cat("gradient_coefficients_y"),
        limiter_cells=lim_cells, limiter_dx=lim_dx, limiter_dy=lim_dy,
        parabolic_sources=cat("parabolic_sources", "cell").astype(np.int64),
        parabolic_neighbours=cat("parabolic_neighbours", "cell").astype(np.int64),
        parabolic_dx=cat("parabolic_dx"), parabolic_dy=cat("parabolic_dy"),
    )
    return geo, BatchLayout(cells.astype(np.int64), faces.astype(np.int64), len(geometries))


# ------------------------------------------------------------------- stepper


class BatchStepper:
    """Explicit steps of a batch with one global time step per case."""

    def __init__(self, dg: DeviceGeometry, layout: BatchLayout, settings, mode: str = "fast"):
        """The stage kernels' launch shapes can be tuned for the batch with
        ``dg.autotune(U, stepper.cfg)`` before :meth:`capture`."""
        self.dg = dg
        self.layout = layout
        self.cfg = make_config(settings, mode)
        self.scheme = TIME_SCHEME_CODES[settings.time_integration]
        dev = dg.device
        self.offsets = torch.as_tensor(layout.cell_offsets.astype(np.int32), device=dev)
        self.dt_case = torch.empty(layout.n_cases, dtype=torch.float64, device=dev)
        self.dt_cells = torch.empty(dg.n_cells, dtype=torch.float64, device=dev)
        self.graph = None
        self.graph_steps = 0

    def step(self, U: torch.Tensor) -> None:
        """One step of every case (no host synchronisation)."""
        lib, h = self.dg.lib, self.dg.handle
        s = _stream_ptr()
        P = self.dg.primitive(U, self.cfg, out=self.dg.primitive_buffer())
        lib.check(lib.mcfd_batch_time_steps(h, C.byref(self.cfg), P.data_ptr(), self.offsets.data_ptr(),
                                            self.layout.n_cases, self.dt_case.data_ptr(), self.dt_cells.data_ptr(),
                                            s), "mcfd_batch_time_steps")
        self.dg.explicit_step(U, self.cfg, self.scheme, self.dt_cells)

    def capture(self, U: torch.Tensor, steps: int) -> None:
        """Capture ``steps`` batch steps into one CUDA graph (U is updated in
        place on every replay)."""
        stream = torch.cuda.Stream(device=self.dg.device)
        stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(stream):
            self.step(U)  # warm up outside capture
        torch.cuda.current_stream().wait_stream(stream)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            for _ in range(steps):
                self.step(U)
        self.graph = g
        self.graph_steps = steps

    def replay(self) -> None:
        self.graph.replay()


def build_batch(cases, device=None):
    geoms = [build_geometry(case.mesh, case) for case, _ in cases]
    geo, layout = concatenate(geoms)
    P0 = np.concatenate([P for _, P in cases])
    return geo, layout, P0, geoms
