"""Benchmark: FP64 RK3 HLLC-MUSCL step throughput (cell-updates/s) on GB300.

Workload (default): the isentropic vortex on a periodic [0,10]^2 box of
1024x1024 quads with a seed-chosen half split into triangles (1,572,864 mixed
cells), HLLC flux, MUSCL-linear reconstruction with the Venkatakrishnan
limiter, SSP-RK3, CFL 0.8, global adaptive time step.  One "step" is one full
reference time step: the stable time step (min over cells) and the three RK3
stages (reconstruct, face flux, cell gather + stage update), all on the
device.  Inputs are synthetic (seeded); the working set (~1.2 GB) is far
larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

``--impl reference`` times the oracle (the C restatement of the reference's
single-threaded CPU path) on the host cores for the same workload.
"""

from __future__ import annotations

import argparse
import contextlib
import ctypes as C
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "RK3 HLLC-MUSCL cell-updates/s"
UNIT = "cell-updates/s"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gpu", "reference"), default="gpu")
    ap.add_argument("--workload", default="vortex1024",
                    choices=("vortex1024", "vortex1024all", "vortex512", "vortex512all", "vortex256", "batch256",
                             "adjoint", "bump"))
    ap.add_argument("--checkpoint-every", type=int, default=20)
    ap.add_argument("--batch-adjoint-steps", type=int, default=20)
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--launch-shapes", default="",
                    help="set the stage kernels' launch shapes instead of autotuning: reconstruction threads, flux "
                         "threads, flux faces per thread, gather threads, per-variable reconstruction (0/1), "
                         "e.g. 64,64,1,64,1 (mcfd_set_launch_shapes)")
    ap.add_argument("--batch-adjoint-checkpoint", type=int, default=5)
    ap.add_argument("--batch-cases", type=int, default=256)
    ap.add_argument("--graph-steps", type=int, default=10)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=10,
                    help="RK3 steps of the CPU baseline sample (about 12 s on one Grace core); the device state "
                         "after the same steps is compared with it")
    ap.add_argument("--profile-steps", type=int, default=3)
    ap.add_argument("--mode", choices=("fast", "exact", "fma"), default="fast",
                    help="exact: reference operation order, bit-exact; fast: exact arithmetic with the "
                         "limiter minimum through the smallest ratio; fma: shared reciprocals + FMA "
                         "(outside the 1e-12 bar on fine meshes)")
    ap.add_argument("--parity-steps", type=int, default=10)
    ap.add_argument("--variant-steps", type=int, default=20)
    ap.add_argument("--exact-steps", type=int, default=100,
                    help="steps of the run compared with the exactly translated vortex")
    ap.add_argument("--extras", default="alltri,adjoint,batch",
                    help="comma list of the sub-measurements of the default run: alltri (the 2,097,152-cell "
                         "all-triangle mesh), adjoint (O-grid adjoint / forward cost), batch (256 uneven cases); "
                         "'none' for none")
    ap.add_argument("--budget-s", type=float, default=600.0,
                    help="bump workload: wall-clock budget of the implicit step (checked between GMRES calls)")
    ap.add_argument("--bump-size", default="512x256")
    ap.add_argument("--bump-steps", type=int, default=1)
    ap.add_argument("--bump-until-drop", type=float, default=0.0,
                    help="bump workload: stop once the density residual has fallen by this factor (1e-8 for the "
                         "configuration's 8 orders); progress lines go to stderr and --bump-log")
    ap.add_argument("--bump-log", default="",
                    help="bump workload: file rewritten with the line so far after every step")
    ap.add_argument("--bump-oracle", action="store_true",
                    help="bump workload: also run the oracle's SciPy restatement of the same step and compare")
    ap.add_argument("--numbering", choices=("generator", "random", "rcm", "random-rcm-cells"), default="generator",
                    help="vortex workloads: cell and face ids as generated, randomly permuted (as a mesh file "
                         "may number them), renumbered by reverse Cuthill-McKee, or randomly permuted and then "
                         "its cells (not its faces) renumbered by reverse Cuthill-McKee (meshes.renumber_cells, "
                         "which keeps every cell's results bit for bit)")
    return ap.parse_args(argv)


WORKLOADS = {
    "vortex1024": dict(n=1024, split="half"),
    "vortex1024all": dict(n=1024, split="all"),
    "vortex512": dict(n=512, split="half"),
    "vortex512all": dict(n=512, split="all"),
    "vortex256": dict(n=256, split="half"),
}


def _sample_case(name, n, host=None, numbering="generator"):
    """(case, settings, geometry, initial primitive) of workload ``name``,
    at ``n`` x ``n`` quads when given, with the mesh's ids as generated,
    randomly permuted (seed 7) or renumbered by reverse Cuthill-McKee."""
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import (cell_centroids, permute_mesh, renumber_cells, reverse_cuthill_mckee,
                                      vortex_case, vortex_primitive)

    w = WORKLOADS[name]
    case, _ = vortex_case(n or w["n"], split=w["split"])
    if numbering == "random":
        rng = np.random.default_rng(7)
        case.mesh = permute_mesh(case.mesh, rng.permutation(len(case.mesh.cells)),
                                 rng.permutation(len(case.mesh.faces)))
    elif numbering == "rcm":
        case.mesh = permute_mesh(case.mesh, *reverse_cuthill_mckee(case.mesh))
    elif numbering == "random-rcm-cells":
        rng = np.random.default_rng(7)
        case.mesh = permute_mesh(case.mesh, rng.permutation(len(case.mesh.cells)),
                                 rng.permutation(len(case.mesh.faces)))
        case.mesh, cell_order = renumber_cells(case.mesh)
        g = build_geometry(case.mesh, case, host=host)
        return case, case.numerics, g, vortex_primitive(cell_centroids(case.mesh))
    g = build_geometry(case.mesh, case, host=host)
    return case, case.numerics, g, vortex_primitive(cell_centroids(case.mesh))


def make_workload(name, host=None, numbering="generator"):
    """The workload's case, settings, geometry, initial primitive state and
    the ``config`` both arms print (identical keys and values; the kernel
    variant of the device arm is the line's separate ``mode`` key).  ``host``:
    the cell / face geometry loops to build with (the CPU reference arm passes
    the oracle's, so that it never loads the product library)."""
    w = WORKLOADS[name]
    case, settings, g, P0 = _sample_case(name, w["n"], host=host, numbering=numbering)
    config = {
        "workload": f"isentropic vortex, periodic [0,10]^2, {w['n']}x{w['n']} quads, "
                    f"{'half' if w['split'] == 'half' else 'all'} split to triangles, jitter 0.15h, seed 0"
                    + ("" if numbering == "generator" else f", ids {numbering}"),
        "cells": int(len(g.areas)),
        "faces": int(len(g.face_lengths)),
        "interior_faces": int(len(g.interior_faces)),
        "periodic_pairs": int(len(g.periodic_faces_a)),
        "flux": settings.flux, "reconstruction": settings.reconstruction, "limiter": settings.limiter,
        "time_integration": settings.time_integration, "cfl": settings.cfl,
        "time_step_mode": settings.time_step_mode, "precision": "fp64",
        "l2": "inputs larger than L2 (working set > 1 GB), no flush",
        "parallelism": "replicas",
    }
    return case, settings, g, P0, config


def model_bytes(g):
    """Algorithmic bytes per launch group of each kernel class (the
    reference 3-pass model: every array the reference algorithm produces or
    consumes moves once).  C cells, F flux faces, E gradient entries, L
    limiter entries."""
    C = len(g.areas)
    F = len(g.interior_faces) + len(g.periodic_faces_a) + len(g.wall_faces) + len(g.velocity_inlet_faces) \
        + len(g.pressure_outlet_faces) + len(g.far_field_faces)
    E = len(g.gradient_sources)
    L = len(g.limiter_cells)
    return {
        "reconstruct": C * (32 + 64 + 32) + E * (4 + 16) + L * 16,
        "flux": C * (32 + 64 + 32) + F * (8 + 16 + 8 + 32 + 32),
        "gather": C * (32 + 32 + 32 + 8) + F * 32,
        "time_step": C * (32 + 8) + F * (8 + 16 + 8),
        "primitive": C * 64,
    }, dict(C=C, F=F, E=E, L=L)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit()) if rows else None}


def measured_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        d = json.loads(path.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_oracle_run(g, settings, P0, steps):
    """The oracle (C restatement of the reference path, one thread) on the same
    mesh: ``steps`` full RK3 steps including the stable time step.  Returns
    (cell-updates/s, seconds, final state, physical time reached)."""
    from oracle.oracle import Oracle

    orc = Oracle(g)
    U = orc.conservative(P0, settings.gamma)
    orc.solve(U, settings, 1)  # warm caches / page-in
    t0 = time.perf_counter()
    UN, t_end = orc.solve(U, settings, steps)
    dt = time.perf_counter() - t0
    return len(g.areas) * steps / dt, dt, UN, t_end


def oracle_residual(g, settings, U):
    from oracle.oracle import Oracle

    return Oracle(g).residual(U, settings)


def max_rel(a, b) -> float:
    """max |a - b| / max |b| over all entries (0 when both are zero)."""
    a, b = np.asarray(a), np.asarray(b)
    den = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / den if den > 0 else float(np.max(np.abs(a - b)))


# CPU time the reference arm may spend on its timed and warm-up steps, at a
# conservative one-core rate of the reference path (cell-updates/s)
REFERENCE_BUDGET_S, REFERENCE_RATE = 180.0, 1.0e6


def reference_sample(name, steps, warmup):
    """The workload the reference arm times: the named one, or the same
    recipe at the largest smaller size whose ``steps + warmup`` full RK3
    steps fit the CPU budget (the per-cell rate does not depend on the size
    once the mesh exceeds the caches)."""
    w = WORKLOADS[name]
    for n in (w["n"], 512, 256):
        if n > w["n"]:
            continue
        cells = n * n * (3 if w["split"] == "half" else 4) // 2
        if cells * (steps + warmup) / REFERENCE_RATE <= REFERENCE_BUDGET_S:
            break
    return n


def run_reference(args):
    """The reference arm: the reference's CPU path (its C restatement, one
    thread) on the host.  It builds the mesh geometry with the oracle's own
    restatement of the reference's geometry loops, so nothing of the product
    library is loaded in this process."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload not in WORKLOADS:
        print(json.dumps({"impl": "reference", "unavailable": f"workload {args.workload} has no CPU reference arm; "
                                                             "its line compares against the oracle itself"}))
        return
    from oracle.oracle import GeometryHost, Oracle

    host = GeometryHost()
    case, settings, g, P0, config = make_workload(args.workload, host=host)
    steps, warm = args.steps, args.warmup
    n = reference_sample(args.workload, steps, warm)
    if n != WORKLOADS[args.workload]["n"]:
        case, settings, g, P0 = _sample_case(args.workload, n, host=host)
    orc = Oracle(g)
    U = orc.conservative(P0, settings.gamma)
    U, _ = orc.solve(U, settings, warm)
    t0 = time.perf_counter()
    orc.solve(U, settings, steps)
    elapsed = time.perf_counter() - t0
    value = len(g.areas) * steps / elapsed
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * elapsed / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded vortex)",
        "config": config, "mode": "reference operation order (CPU)",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"{steps} RK3 steps of the same recipe at {n}x{n} quads ({len(g.areas)} "
                                   f"cells{'' if n == WORKLOADS[args.workload]['n'] else ', reduced to fit ~3 min of CPU time'})"
                                   " (oracle: single-threaded C restatement of the reference path, geometry "
                                   "included; the reference itself is single-threaded NumPy/Numba)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def replica_throughput(ms_local, cells, steps, dist=None, device=None):
    """The replica job's time and throughput: every rank steps its own copy
    of the workload (no data-path collective), the job's time is the slowest
    rank's (MAX over ranks), and the value counts every rank's cells:
    world * cells * steps / time.  Returns (ms, cell-updates/s)."""
    import torch

    world = 1
    ms = float(ms_local)
    if dist is not None:
        world = dist.get_world_size()
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t)
    return ms, world * cells * steps / (ms * 1e-3)


def _ncu_summary():
    tpath = ROOT / "profiles" / "ncu_summary.json"
    return json.loads(tpath.read_text()) if tpath.exists() else {}


def reconstruction_fp64_model(g, issued_per_cell=None):
    """FP64 operations per cell that the reference's reconstruction takes in
    its own expression order (_kernels.py:10-67, 71-98, 240-273), counted
    from the mesh's entry counts, against the FP64-pipe instructions the
    device kernel issues (ncu).  Per gradient entry and variable: the
    difference, two products and two sums (5); per limiter entry and
    variable: the increment grad . r (3), the numerator of the ratio (1), the
    ratio and the smooth limiter's quotient (2 divisions) and the rest of its
    rational function (7); per variable the tolerance (1); per face state
    and variable the increment again, the factor's product and the sum (5).
    A division issued by the FP64 unit takes ~8.6 FP64-pipe slots on GB300
    (measured by tests/arith_throughput.cu)."""
    C = len(g.areas)
    e = len(g.gradient_sources) / C
    l = len(g.limiter_cells) / C
    arithmetic = 4 * (5 * e + (3 + 1 + 7) * l + 1 + 5 * l)
    divisions = 4 * 2 * l
    out = {"reference_operations_per_cell": arithmetic + divisions, "of_which_divisions": divisions,
           "fp64_pipe_slots_per_cell_if_native": arithmetic + 8.6 * divisions,
           "gradient_entries_per_cell": e, "limiter_entries_per_cell": l,
           "issued_fp64_instructions_per_cell": issued_per_cell,
           "how": "divisions and square roots on the integer pipe (the same IEEE results), gradient and face "
                  "products on the integer pipe, the limiter minimum through each variable's smallest ratio "
                  "(3 divisions per variable instead of 2 per entry), increments kept for the face states, the "
                  "first sum term without an FP64 addition"}
    if issued_per_cell:
        out["issued_over_reference_operations"] = issued_per_cell / (arithmetic + divisions)
    return out


def roofline_for(name, g, kernels, ms_per_step, mode):
    """The HBM roofline of the dominant kernel (algorithmic bytes of the
    reference 3-pass model per launch over its live launch time), the step's
    figure against the same model, and the FP64 side of the dominant kernel
    (its FP64 instructions per cell, counted by ncu on the same recipe, over
    the live launch time, against the measured FP64 issue rate)."""
    C = len(g.areas)
    mbytes, _ = model_bytes(g)
    dominant = max(kernels, key=lambda k: kernels[k]["ms_total"])
    peak, peak_kind = measured_peaks()
    achieved = mbytes[dominant] / (kernels[dominant]["ms_per_group"] * 1e-3) / 1e9
    summary = _ncu_summary()
    recipe = summary.get("recipes", {}).get(WORKLOADS[name]["split"], {}) if name in WORKLOADS else {}
    traffic = fp64 = None
    fp64_pipe = recipe.get("fp64_pipe_active_pct", {}).get(dominant)
    alu_pipe = recipe.get("alu_pipe_active_pct", {}).get(dominant)
    issue = recipe.get("issue_active_pct", {}).get(dominant)
    per_cell = recipe.get("dram_bytes_per_cell", {}).get(dominant)
    if per_cell:
        traffic = per_cell * C  # ncu capture on the 512^2 mesh of this recipe, scaled by cells
    ipc = recipe.get("fp64_instructions_per_cell", {}).get(dominant)
    fpeak = summary.get("fp64_peak_ginstr_s")
    if ipc and fpeak and mode == recipe.get("mode"):
        got = ipc * C / (kernels[dominant]["ms_per_group"] * 1e-3) / 1e9
        fp64 = {"achieved": got, "peak": fpeak, "unit": "G FP64 thread-instructions/s", "frac": got / fpeak,
                "instructions_per_cell": ipc,
                "source": "instructions per cell from the ncu capture of this kernel on the 512^2 mesh of this "
                          "recipe; peak: " + summary.get("fp64_peak_source", "")}
    step_bytes = 3 * (mbytes["reconstruct"] + mbytes["flux"] + mbytes["gather"]) - 32 * C + mbytes["time_step"]
    return {
        "bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
        "algorithmic_bytes_per_launch": mbytes[dominant],
        "step_algorithmic_bytes_per_cell": step_bytes / C,
        "step_achieved_gbs": step_bytes / (ms_per_step * 1e-3) / 1e9,
        "step_frac": step_bytes / (ms_per_step * 1e-3) / 1e9 / peak,
        "fp64_pipe_active_pct_ncu": fp64_pipe,
        "alu_pipe_active_pct_ncu": alu_pipe,
        "issue_active_pct_ncu": issue,
        "fp64": fp64,
        "fp64_model": reconstruction_fp64_model(g, ipc) if dominant == "reconstruct" else None,
        "note": ("compute bound, not HBM bound: GB300's FP64 pipe issues ~0.5 T instr/s; divisions, square roots "
                 "and part of the products run bit-identically on the integer pipe, and ncu shows the dominant "
                 "kernel sharing the FP64 and ALU pipes (fp64 / alu / issue percentages above); 'fp64' is the "
                 "kernel's FP64 instruction rate against the measured FP64 issue rate"),
    }


def _barrier(dist=None):
    import torch

    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()


class ExplicitRun:
    """One vortex workload on the device: geometry handle, initial state and
    the RK3 step of the bench's kernel variant."""

    def __init__(self, name, args, device):
        import torch

        from meshcfd_gb300.device import DeviceGeometry, make_config, primitive_to_conservative

        self.name, self.args, self.device = name, args, device
        self.case, self.settings, self.g, self.P0, self.config = make_workload(name, numbering=args.numbering)
        self.cfg = make_config(self.settings, mode=args.mode)
        self.dg = DeviceGeometry(self.g, device)
        self.C = self.dg.n_cells
        self.U_init = primitive_to_conservative(self.P0, self.settings.gamma)
        self.U = torch.as_tensor(self.U_init, device=device)
        self.dt = torch.empty(1, dtype=torch.float64, device=device)
        self.dt_next = torch.empty(1, dtype=torch.float64, device=device)
        self.P = self.dg.primitive_buffer()
        self.primed = None  # the settings whose time step self.dt holds for the state in self.U
        self.tuned = None

    def step(self, cfg=None):
        """One step of the run's state: the stable time step, then the RK3
        stages.  Once primed (``reset``), the time step of every step comes
        from the previous step's last stage (mcfd_explicit_step_next, the
        values mcfd_time_steps gives) and the step starts from the primitive
        that stage left; ``self.last_dt`` is the step's time step."""
        cfg = self.cfg if cfg is None else cfg
        if self.primed is not cfg:
            self.dg.time_steps(self.P, cfg, out_min=self.dt)
            self.primed = cfg
        self.dg.explicit_step_next(self.U, cfg, 2, self.dt, next_dt_min=self.dt_next, primitive_current=True)
        self.last_dt = self.dt
        self.dt, self.dt_next = self.dt_next, self.dt

    def step_plain(self):
        """One drop-in step of the state in self.U: primitive, stable time
        step and RK3 stages, each from the state (mcfd_primitive,
        mcfd_time_steps, then mcfd_explicit_step_next starting from that
        primitive, without a look-ahead)."""
        self.dg.primitive(self.U, self.cfg, out=self.P)
        self.dg.time_steps(self.P, self.cfg, out_min=self.dt)
        self.dg.explicit_step_next(self.U, self.cfg, 2, self.dt, primitive_current=True)
        self.primed = None

    def reset(self, cfg=None):
        import torch

        self.U.copy_(torch.as_tensor(self.U_init, device=self.device))
        self.dg.primitive(self.U, cfg or self.cfg, out=self.P)
        self.primed = None

    def march(self, steps, cfg=None):
        """``steps`` steps from the initial state; returns the physical time."""
        self.reset(cfg)
        t = 0.0
        for _ in range(steps):
            self.step(cfg=cfg)
            t += float(self.last_dt.item())
        self.dg.check_status()
        return t

    def measure(self, steps, warmup, dist=None, world=1, clocks=True):
        """Warm-up, then ``steps`` timed steps bracketed by barriers (CUDA
        events on the launching stream); per-kernel times from the library's
        own events over ``--profile-steps`` more steps; the roofline."""
        import torch

        from meshcfd_gb300 import _lib

        native = _lib.native()
        stream = torch.cuda.current_stream()
        self.reset()
        if self.args.launch_shapes:
            shapes = [int(v) for v in self.args.launch_shapes.split(",")]
            self.dg.lib.check(self.dg.lib.mcfd_set_launch_shapes(self.dg.handle, (C.c_int32 * 5)(*shapes)),
                              "mcfd_set_launch_shapes")
            self.tuned = dict(zip(("reconstruct_threads", "flux_threads", "flux_faces_per_thread", "gather_threads",
                                   "reconstruct_per_variable"), shapes))
        else:
            self.tuned = self.dg.autotune(self.U, self.cfg) if not self.args.no_autotune else None
        self.reset()
        for _ in range(warmup):
            self.step()
        self.dg.check_status()
        _barrier(dist)
        launches0 = native.mcfd_launch_count()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sampler = ClockSampler(self.device.index) if clocks else None
        with sampler or contextlib.nullcontext():
            start.record(stream)
            for _ in range(steps):
                self.step()
            stop.record(stream)
            _barrier(dist)
        launches = native.mcfd_launch_count() - launches0
        ms, value = replica_throughput(start.elapsed_time(stop), self.C, steps, dist, self.device)
        self.dg.check_status()
        ms_per_step = ms / steps
        native.mcfd_profile_enable(self.dg.handle, 1)
        for _ in range(self.args.profile_steps):
            self.step()
        tot = (C.c_double * 6)()
        grp = (C.c_int64 * 6)()
        native.mcfd_profile_read(self.dg.handle, tot, grp)
        native.mcfd_profile_enable(self.dg.handle, 0)
        names = ("primitive", "reconstruct", "flux", "gather", "time_step", "other")
        kernels = {names[k]: {"ms_total": tot[k], "groups": int(grp[k]),
                              "ms_per_group": tot[k] / grp[k] if grp[k] else None} for k in range(6) if grp[k]}
        total_ms = sum(v["ms_total"] for v in kernels.values())
        for v in kernels.values():
            v["share"] = v["ms_total"] / total_ms
        return {"value": value, "ms_per_step": ms_per_step, "launches": int(launches),
                "clocks": sampler.summary() if clocks else None, "kernels": kernels,
                "roofline": roofline_for(self.name, self.g, kernels, ms_per_step, self.args.mode) if kernels else None,
                "autotune": self.tuned}

    def vs_oracle(self, steps):
        """The oracle's ``steps`` steps from the initial state (timed: the CPU
        baseline) against the device's, plus one residual of the initial
        state: max-norm errors relative to the oracle's values."""
        rate, secs, UN, t_ref = cpu_oracle_run(self.g, self.settings, self.P0, steps)
        t_dev = self.march(steps)
        err_state = max_rel(self.U.cpu().numpy(), UN)
        import torch

        R = self.dg.residual(torch.as_tensor(self.U_init, device=self.device), self.cfg)
        self.dg.check_status()
        err_res = max_rel(R.cpu().numpy(), oracle_residual(self.g, self.settings, self.U_init))
        cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{steps} RK3 steps of the same {self.C}-cell workload in {secs:.1f} s "
                         "(oracle: single-threaded C restatement of the reference path)"}
        vs = {"reference": "oracle (C restatement of the reference path, pinned to reference-made fixtures)",
              "mode": self.args.mode, "steps": steps, "state_max_rel_err": err_state,
              "residual_max_rel_err": err_res, "time_rel_err": abs(t_dev - t_ref) / t_ref,
              "bar": {"residual": 1e-12, "state_after_100_steps": 1e-9}}
        return cpu, vs

    def exact_vortex_error(self, steps):
        """Density after ``steps`` steps against the exactly translated vortex
        at the time reached: area-weighted relative L2 error and max error."""
        from meshcfd_gb300.meshes import cell_centroids, vortex_primitive

        t = self.march(steps)
        rho = self.U[:, 0].cpu().numpy()
        exact = vortex_primitive(cell_centroids(self.case.mesh), t=t)[:, 0]
        a = np.asarray(self.g.areas)
        l2 = math.sqrt(float(np.sum(a * (rho - exact) ** 2)) / float(np.sum(a * exact ** 2)))
        dip = math.sqrt(float(np.sum(a * (rho - exact) ** 2)) / float(np.sum(a * (exact - 1.0) ** 2)))
        return {"steps": steps, "time": t, "density_l2_rel_err": l2, "density_l2_err_rel_to_vortex_dip": dip,
                "density_max_abs_err": float(np.max(np.abs(rho - exact))), "mode": self.args.mode}

    def close(self):
        self.dg.close()


def run_gpu(args):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    from meshcfd_gb300.device import make_config

    run = ExplicitRun(args.workload, args, device)
    main = run.measure(args.steps, args.warmup, dist, world)
    C, cfg, stream, config = run.C, run.cfg, torch.cuda.current_stream(), run.config

    # end to end through the public API: state in pinned host memory, H2D +
    # primitive + step + D2H every step
    e2e = None
    if not args.no_e2e:
        host = torch.as_tensor(run.U_init).pin_memory()
        out = torch.empty_like(host).pin_memory()

        def e2e_step():
            run.U.copy_(host, non_blocking=True)
            run.step_plain()
            out.copy_(run.U, non_blocking=True)

        for _ in range(2):
            e2e_step()
        _barrier(dist)
        s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s2.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e2.record(stream)
        _barrier(dist)
        ms2, e2e_value = replica_throughput(s2.elapsed_time(e2), C, args.steps, dist, device)
        run.dg.check_status()
        e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(host.numel() * 8),
               "d2h_bytes_per_step": int(out.numel() * 8), "ms_per_step": ms2 / args.steps}

    extras = set() if args.extras == "none" else set(args.extras.split(","))
    parity = cpu = vs_oracle = exact_err = alltri = adjoint = batch = None
    variants = {}
    if world == 1:
        # this run's kernels against the bit-exact variant on the device: one
        # residual and --parity-steps steps from the initial state
        if args.parity_steps > 0:
            cfg_exact = make_config(run.settings, mode="exact")
            U0 = torch.as_tensor(run.U_init, device=device)
            Ra, Rb = run.dg.residual(U0, cfg), run.dg.residual(U0, cfg_exact)
            res_err = float((Ra - Rb).abs().max() / Rb.abs().max())
            run.march(args.parity_steps, cfg_exact)
            Ub = run.U.clone()
            run.march(args.parity_steps)
            parity = {"reference": "the bit-exact variant on the device", "residual_max_rel_err": res_err,
                      "steps": args.parity_steps, "state_max_rel_err": float((run.U - Ub).abs().max() / Ub.abs().max())}
        # the other kernel variants: step time and residual deviation from exact
        if args.variant_steps > 0:
            cfg_exact = make_config(run.settings, mode="exact")
            U0 = torch.as_tensor(run.U_init, device=device)
            Rb = run.dg.residual(U0, cfg_exact)
            for mode in ("exact", "fast", "fma"):
                cf = make_config(run.settings, mode=mode)
                err = float((run.dg.residual(U0, cf) - Rb).abs().max() / Rb.abs().max())
                run.reset(cf)
                for _ in range(2):
                    run.step(cfg=cf)
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                for _ in range(args.variant_steps):
                    run.step(cfg=cf)
                b.record(stream)
                torch.cuda.synchronize()
                msv = a.elapsed_time(b) / args.variant_steps
                variants[mode] = {"ms_per_step": msv, "value": C / (msv * 1e-3), "residual_max_rel_err": err}
            run.dg.check_status()
        if rank == 0 and not args.no_cpu_baseline and args.cpu_steps > 0:
            cpu, vs_oracle = run.vs_oracle(args.cpu_steps)
        if args.exact_steps > 0 and args.workload in WORKLOADS:
            exact_err = run.exact_vortex_error(args.exact_steps)
    run.close()
    del run
    torch.cuda.empty_cache()
    if world == 1 and rank == 0:
        if "alltri" in extras and args.workload == "vortex1024":
            alltri = measure_alltri(args, device)
        if "adjoint" in extras:
            adjoint = adjoint_measure(args, device, steps=400)
        if "batch" in extras:
            batch = batch_measure(args, device, steps=20)
    if rank == 0:
        line = {
            "metric": METRIC, "value": main["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": main["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded vortex mesh and state)",
            "config": config, "mode": args.mode, "gpu_launches": main["launches"],
            "roofline": main["roofline"], "kernels": main["kernels"], "autotune": main["autotune"],
            "e2e": e2e, "cpu_baseline": cpu, "vs_oracle": vs_oracle,
            "vs_oracle_max_rel_err": vs_oracle["state_max_rel_err"] if vs_oracle else None,
            "clocks": main["clocks"], "parity": parity, "variants": variants, "vortex_exact_err": exact_err,
            "all_tri": alltri, "adjoint_over_forward": adjoint["adjoint_over_forward"] if adjoint else None,
            "adjoint": adjoint,
            "batched_over_one_at_a_time": batch["batched_over_one_at_a_time"] if batch else None,
            "batch": batch,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def measure_alltri(args, device):
    """The all-triangle 1024^2 vortex (2,097,152 cells): timed steps, roofline,
    and the oracle over a few steps."""
    import torch

    run = ExplicitRun("vortex1024all", args, device)
    m = run.measure(args.steps, args.warmup, clocks=False)
    out = {"cells": run.C, "config": run.config, "value": m["value"], "unit": UNIT,
           "ms_per_step": m["ms_per_step"], "steps": args.steps, "roofline": m["roofline"], "kernels": m["kernels"],
           "gpu_launches": m["launches"]}
    if not args.no_cpu_baseline:
        cpu, vs = run.vs_oracle(min(3, max(1, args.cpu_steps)))
        out["cpu_baseline"], out["vs_oracle"] = cpu, vs
    run.close()
    del run
    torch.cuda.empty_cache()
    return out


def batch_measure(args, device, steps, clocks=True):
    """The seeded 256 uneven channel/Riemann cases (HLLC, MUSCL-Venkatakrishnan,
    RK3), all cases in one geometry with one launch per kernel per stage,
    steps captured in a CUDA graph, against the same cases solved one at a
    time with the plain path (host loop per case); plus the batched adjoint."""
    import torch

    from meshcfd_gb300.batch import BatchStepper, batch_workload, build_batch
    from meshcfd_gb300.device import DeviceGeometry, primitive_to_conservative
    from meshcfd_gb300.solver import run_explicit

    t0 = time.perf_counter()
    cases = batch_workload(n_cases=args.batch_cases)
    geo, layout, P0, geoms = build_batch(cases)
    settings = cases[0][0].numerics
    U0 = primitive_to_conservative(P0, settings.gamma)
    dg = DeviceGeometry(geo, device)
    setup_s = time.perf_counter() - t0
    stepper = BatchStepper(dg, layout, settings, mode=args.mode)
    U = torch.as_tensor(U0, device=device)
    tuned = dg.autotune(U, stepper.cfg) if not args.no_autotune else None
    gsteps = max(1, min(args.graph_steps, steps))
    stepper.capture(U, gsteps)
    for _ in range(max(1, args.warmup // gsteps)):
        stepper.replay()
    torch.cuda.synchronize()
    U.copy_(torch.as_tensor(U0, device=device))
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(1, steps // gsteps)
    sampler = ClockSampler(device.index) if clocks else None
    with sampler or contextlib.nullcontext():
        a.record()
        for _ in range(reps):
            stepper.replay()
        b.record()
        torch.cuda.synchronize()
    dg.check_status()
    batched_ms = a.elapsed_time(b)
    done_steps = reps * gsteps
    U_launches = U.clone()
    # the same steps with each stage as one cooperative launch (grid barriers
    # between reconstruction, fluxes and gather), captured the same way
    dg.set_fused_stage(True)
    fused_stepper = BatchStepper(dg, layout, settings, mode=args.mode)
    U.copy_(torch.as_tensor(U0, device=device))
    fused_stepper.capture(U, gsteps)
    for _ in range(max(1, args.warmup // gsteps)):
        fused_stepper.replay()
    torch.cuda.synchronize()
    U.copy_(torch.as_tensor(U0, device=device))
    a.record()
    for _ in range(reps):
        fused_stepper.replay()
    b.record()
    torch.cuda.synchronize()
    dg.check_status()
    fused_ms = a.elapsed_time(b)
    fused = {"ms": fused_ms, "cell_updates_per_s": int(dg.n_cells) * done_steps / (fused_ms * 1e-3),
             "resident_blocks_per_sm": dg.fused_stage_blocks,
             "bit_identical_to_launch_per_kernel": bool(torch.equal(U, U_launches))}
    dg.set_fused_stage(False)
    del fused_stepper
    stage_launch = "one cooperative launch per stage" if fused_ms < batched_ms else "one launch per kernel"
    per_kernel_ms = batched_ms
    batched_ms = min(batched_ms, fused_ms)
    U.copy_(U_launches)
    # one at a time: the plain path per case (its own geometry handle and loop)
    singles = [DeviceGeometry(g, device) for g in geoms]
    Us = [torch.as_tensor(U0[layout.cell_offsets[k]:layout.cell_offsets[k + 1]], device=device)
          for k in range(layout.n_cases)]
    settings.max_iterations = done_steps
    torch.cuda.synchronize()
    a2, b2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a2.record()
    for dgk, Uk in zip(singles, Us):
        run_explicit(dgk, settings, Uk, mode=args.mode, final_residual=False)
    b2.record()
    torch.cuda.synchronize()
    single_ms = a2.elapsed_time(b2)
    # both paths agree bit for bit
    Ub = U.cpu().numpy()
    same = all(np.array_equal(Ub[layout.cell_offsets[k]:layout.cell_offsets[k + 1]], Us[k].cpu().numpy())
               for k in range(layout.n_cases))
    for dgk in singles:
        dgk.close()
    n_cells = int(dg.n_cells)
    adjoint = None
    if args.batch_adjoint_steps > 0:
        adjoint = batched_adjoint(dg, layout, settings, U0, stepper, args)
    dg.close()
    return {
        "workload": f"{layout.n_cases} channel/Riemann cases, cells log-uniform [2k,200k], aspect U[1,4], "
                    f"Mach U[0.3,2.0], seed 3", "cells_total": n_cells, "mode": args.mode,
        "graph_steps": gsteps, "setup_s": setup_s, "steps": done_steps,
        "case_steps_per_s": layout.n_cases * done_steps / (batched_ms * 1e-3),
        "batched": {"cell_updates_per_s": n_cells * done_steps / (batched_ms * 1e-3), "ms": batched_ms,
                    "stage_launch": stage_launch},
        "launch_per_kernel": {"cell_updates_per_s": n_cells * done_steps / (per_kernel_ms * 1e-3),
                              "ms": per_kernel_ms},
        "launch_per_stage": fused,
        "one_at_a_time": {"case_steps_per_s": layout.n_cases * done_steps / (single_ms * 1e-3), "ms": single_ms},
        "batched_over_one_at_a_time": single_ms / batched_ms,
        "bit_identical": bool(same), "clocks": sampler.summary() if sampler else None,
        "batched_adjoint": adjoint, "autotune": tuned,
    }


def run_batch(args):
    import torch

    device = torch.device("cuda", 0)
    b = batch_measure(args, device, args.steps)
    line = {
        "metric": "batched case-steps/s (RK3 HLLC-MUSCL, 256 uneven cases)", "value": b["case_steps_per_s"],
        "unit": "case-steps/s", "n_gpus": 1, "steps": b["steps"], "warmup": args.warmup,
        "ms_per_step": b["batched"]["ms"] / b["steps"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded channel/Riemann cases)",
        "config": {k: b[k] for k in ("workload", "cells_total", "mode", "graph_steps", "setup_s")},
        **{k: b[k] for k in ("batched", "launch_per_kernel", "launch_per_stage", "one_at_a_time",
                             "batched_over_one_at_a_time", "bit_identical", "clocks", "batched_adjoint", "autotune")},
    }
    print(json.dumps(line))


def batched_adjoint(dg, layout, settings, U0, stepper, args):
    """Every case's wall-force gradient (the y force on its slip walls) by one
    checkpointed RK3 adjoint over the whole batch: each case keeps its own
    fixed time step (the stable step of its initial state), so the steps are
    per cell."""
    import torch

    from meshcfd_gb300.adjoint import WallForceAdjoint

    device = dg.device
    U = torch.as_tensor(U0, device=device)
    stepper_dt = stepper.dt_cells
    P = dg.primitive(U, stepper.cfg, out=dg.primitive_buffer())
    dg.lib.check(dg.lib.mcfd_batch_time_steps(dg.handle, C.byref(stepper.cfg), P.data_ptr(),
                                              stepper.offsets.data_ptr(), layout.n_cases,
                                              stepper.dt_case.data_ptr(), stepper_dt.data_ptr(),
                                              torch.cuda.current_stream().cuda_stream), "mcfd_batch_time_steps")
    dt_cells = stepper_dt.clone()
    steps, every = args.batch_adjoint_steps, args.batch_adjoint_checkpoint
    # the channels' walls are horizontal: the wall force along y
    adj = WallForceAdjoint(dg, settings, dt_cells, direction=(0.0, 1.0), checkpoint_every=every, mode=args.mode,
                           case_offsets=layout.cell_offsets)
    adj.gradient(U, min(2, steps))  # warm-up
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record()
    UN = adj.forward(U, steps)
    ev[1].record()
    J, dJ = adj.functional(UN)
    lam0 = adj.backward(dJ)
    ev[2].record()
    torch.cuda.synchronize()
    J_cases = adj.functional_per_case(UN)
    fwd, bwd = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    return {"steps": steps, "checkpoint_every": every, "forward_ms": fwd, "adjoint_ms": bwd,
            "adjoint_over_forward": bwd / fwd,
            "cases_gradients_per_s": layout.n_cases / ((fwd + bwd) * 1e-3),
            "sum_of_case_forces": float(np.sum(J_cases)), "J_total": J, "grad_norm": float(lam0.norm())}


def adjoint_measure(args, device, steps, clocks=True):
    """O-grid 1024x512 around a cylinder (seed 2, Mach 0.3 free stream, slip
    wall, far field), HLLC / MUSCL-Venkatakrishnan, RK3 with a fixed time step
    for ``steps`` steps, checkpoints every ``--checkpoint-every`` steps; the
    wall pressure force along x at the final state and its gradient with
    respect to the initial state and the far-field states by the discrete
    adjoint, and the adjoint / forward cost ratio."""
    import torch

    from meshcfd_gb300.adjoint import WallForceAdjoint
    from meshcfd_gb300.device import DeviceGeometry, make_config, primitive_to_conservative
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import ogrid_case

    t0 = time.perf_counter()
    case, P0 = ogrid_case(1024, 512, seed=2, mach=0.3)
    g = build_geometry(case.mesh, case)
    setup_s = time.perf_counter() - t0
    settings = case.numerics
    U0 = torch.as_tensor(primitive_to_conservative(P0, settings.gamma), device=device)
    dg = DeviceGeometry(g, device)
    cfg = make_config(settings, args.mode)
    _, dt_min = dg.time_steps(dg.primitive(U0, cfg), cfg)
    dt = 0.9 * float(dt_min)
    adj = WallForceAdjoint(dg, settings, dt, direction=(1.0, 0.0), checkpoint_every=args.checkpoint_every,
                           mode=args.mode)
    for _ in range(max(1, args.warmup)):  # warm-up: a short forward + adjoint
        adj.gradient(U0, min(steps, args.checkpoint_every + 1))
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    before = _launches()
    sampler = ClockSampler(device.index) if clocks else None
    with sampler or contextlib.nullcontext():
        ev[0].record()
        UN = adj.forward(U0, steps)
        ev[1].record()
        J, dJ = adj.functional(UN)
        lam0 = adj.backward(dJ)
        ev[2].record()
        torch.cuda.synchronize()
    launches = _launches() - before
    fwd_ms, adj_ms = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    C = int(dg.n_cells)
    far = float(adj.far_acc.norm())
    fd_check = adjoint_fd_check(dg, case, g, P0, steps, args) if steps >= 400 else None
    out = {
        "workload": f"O-grid 1024x512 around a cylinder ({C} cells), Mach 0.3, HLLC, MUSCL linear, "
                    f"Venkatakrishnan, RK3 fixed dt, {steps} steps, checkpoint every {args.checkpoint_every}",
        "mode": args.mode, "dt": dt, "setup_s": setup_s, "steps": steps, "checkpoint_every": args.checkpoint_every,
        "adjoint_over_forward": adj_ms / fwd_ms,
        "forward": {"ms": fwd_ms, "cell_updates_per_s": C * steps / (fwd_ms * 1e-3)},
        "adjoint": {"ms": adj_ms, "cell_updates_per_s": C * steps / (adj_ms * 1e-3),
                    "work_per_step": "1 replayed RK3 step + 3 residual VJPs"},
        "J": J, "grad_norm": float(lam0.norm()), "far_grad_norm": far,
        "far_grad_note": far_note(P0, settings.gamma, steps * dt) if far == 0.0 else None,
        "fd_check": fd_check,
        "gpu_launches": launches, "clocks": sampler.summary() if sampler else None,
    }
    dg.close()
    return out


def adjoint_fd_check(dg, case, g, P, steps, args):
    """The configuration's gradient check: from the inflow state plus a
    seeded 10 % perturbation, the adjoint gradient of the x wall force in a
    smooth localised initial-state direction (a Gaussian blob upstream of
    the cylinder) against central differences with step 1e-6, with the
    reference's limiter and with the smooth form (K = 5)."""
    import torch

    from meshcfd_gb300.adjoint import WallForceAdjoint
    from meshcfd_gb300.device import primitive_to_conservative

    out = {"steps": steps, "checkpoint_every": args.checkpoint_every, "h": 1e-6,
           "direction": "Gaussian blob (width 0.5) at (-1.5, 0.2) in every variable, scaled by |U|",
           "initial_state": "inflow + seeded 10 % perturbation", "bar": 1e-6}
    rng = np.random.default_rng(11)
    P0 = P + 0.1 * np.array([1.0, 0.3, 0.3, 1.0]) * rng.standard_normal(P.shape)
    U0 = primitive_to_conservative(P0, case.numerics.gamma)
    centers = np.asarray(g.centers).reshape(-1, 2)
    r2 = ((centers - np.array([-1.5, 0.2])) ** 2).sum(axis=1)
    v = np.exp(-r2 / 0.25)[:, None] * np.abs(U0) * np.array([1.0, 0.5, -0.7, 0.8])
    from meshcfd_gb300.device import make_config

    for limiter in ("Venkatakrishnan", "Venkatakrishnan K"):
        case.numerics.limiter = limiter
        case.numerics.venkatakrishnan_k = 5.0
        cfg = make_config(case.numerics, args.mode)
        _, dt_min = dg.time_steps(dg.primitive(torch.as_tensor(U0, device=dg.device), cfg), cfg)
        dt = 0.5 * float(dt_min)
        adj = WallForceAdjoint(dg, case.numerics, dt, direction=(1.0, 0.0), checkpoint_every=args.checkpoint_every,
                               mode=args.mode)
        _, lam0, _ = adj.gradient(torch.as_tensor(U0, device=dg.device), steps)
        vals = [adj.functional(adj.forward(torch.as_tensor(U0 + sg * 1e-6 * v, device=dg.device), steps))[0]
                for sg in (1, -1)]
        fd = (vals[0] - vals[1]) / 2e-6
        an = float((lam0.cpu().numpy() * v).sum())
        out[limiter] = {"adjoint": an, "fd": fd, "rel_err": abs(fd - an) / abs(fd)}
    case.numerics.limiter = "Venkatakrishnan"
    return out


def far_note(P0, gamma, span):
    """Why the far-field gradient of the O-grid wall force is zero over a
    time span: the fastest signal travels (|u| + c) * span, far less than the
    9.5 units between the far-field boundary (half width 10) and the
    cylinder (radius 0.5); the discrete scheme's remaining dependence shrinks
    by the far cells' local CFL number (below 1e-2 there, the time step being
    set by the wall cells) per cell and underflows to exactly zero."""
    rho, u, v, p = np.asarray(P0[-1])
    reach = (math.hypot(u, v) + math.sqrt(gamma * p / rho)) * span
    return (f"identically zero: in {span:.3g} time units a signal from the far field travels {reach:.3g} of the "
            "9.5 units to the wall; the scheme's residual dependence decays by the far cells' local CFL number "
            "per cell and underflows; the inflow gradient is checked on a small box instead")


def run_adjoint(args):
    """Adjoint workload line: the adjoint / forward cost ratio (lower is
    better) at ``--steps`` steps (default 400 here)."""
    import torch

    device = torch.device("cuda", 0)
    steps = args.steps if args.steps != 100 else 400
    a = adjoint_measure(args, device, steps)
    line = {
        "metric": "RK3 wall-force adjoint / forward cost ratio", "value": a["adjoint_over_forward"], "unit": "ratio",
        "n_gpus": 1, "steps": steps, "warmup": args.warmup,
        "ms_per_step": (a["forward"]["ms"] + a["adjoint"]["ms"]) / steps,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded O-grid, free-stream start)",
        "config": {"workload": a["workload"], "mode": a["mode"], "dt": a["dt"], "setup_s": a["setup_s"],
                   "l2_flush": "working set larger than L2"},
        **{k: a[k] for k in ("forward", "adjoint", "J", "grad_norm", "far_grad_norm", "far_grad_note",
                             "gpu_launches", "clocks")},
    }
    print(json.dumps(line))


def run_bump(args):
    """Implicit configuration: the bump channel (circular arc of 10 % chord,
    rows stretched by 1.05 toward the wall, seed 1; Roe, MUSCL linear with
    Barth-Jespersen, implicit Euler with local time steps at CFL 200,
    GMRES(30) to 1e-3 with LU-SGS) at ``--bump-size``, ``--bump-steps``
    implicit steps of the reference's algorithm (time-step halving, Newton,
    line search) on the device under a wall-clock budget.  Reports the
    per-step counts, seconds per step and per GMRES iteration, the density
    residual drop and the state's deviation from the oracle's restatement
    (SciPy GMRES) after the first step when ``--bump-oracle`` is given."""
    import torch

    from meshcfd_gb300.device import DeviceGeometry, make_config, primitive_to_conservative
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.errors import SolverError
    from meshcfd_gb300.implicit import BudgetExceeded, ImplicitEuler
    from meshcfd_gb300.meshes import bump_case

    device = torch.device("cuda", 0)
    nx, ny = (int(v) for v in args.bump_size.split("x"))
    t0 = time.perf_counter()
    case, P0 = bump_case(nx, ny)
    s = case.numerics
    g = build_geometry(case.mesh, case)
    setup_s = time.perf_counter() - t0
    dg = DeviceGeometry(g, device)
    cfg = make_config(s, "exact")
    U0 = primitive_to_conservative(P0, s.gamma)
    U = torch.as_tensor(U0, device=device)
    R = torch.empty_like(U)

    def density_residual():
        dg.residual(U, cfg, out=R)
        dg.check_status()
        return math.sqrt(float((R[:, 0] * R[:, 0]).mean()))

    r0 = density_residual()
    start = time.perf_counter()
    stepper = ImplicitEuler(dg, s, "exact", deadline=start + args.budget_s)
    steps, first_state, first_dt = [], None, None
    status = "completed"
    before = _launches()
    with ClockSampler(device.index) as clocks:
        for k in range(args.bump_steps):
            P = dg.primitive(U, cfg, out=dg.primitive_buffer())
            dt, _ = dg.time_steps(P, cfg, per_cell=True)
            dg.check_status()
            counts0 = (stepper.attempts, stepper.newton_iterations, stepper.gmres_iterations, stepper.gmres_calls,
                       stepper.gmres_seconds)
            ts = time.perf_counter()
            try:
                new, used = stepper.step(U, dt)
            except BudgetExceeded:
                status = f"stopped by the {args.budget_s:.0f} s budget during step {k + 1}"
                break
            except SolverError as error:  # the reference's own stop (solver.py:1363-1368, 810-811)
                status = f"Solver failed at step {k + 1}: {error}"
                break
            torch.cuda.synchronize()
            wall = time.perf_counter() - ts
            if k == 0:
                first_dt = dt.cpu().numpy()
            U.copy_(new)
            if k == 0:
                first_state = U.cpu().numpy()
            r = density_residual()
            gi = stepper.gmres_iterations - counts0[2]
            steps.append({"step": k + 1, "seconds": wall, "halvings": stepper.attempts - counts0[0] - 1,
                          "newton_iterations": stepper.newton_iterations - counts0[1], "gmres_iterations": gi,
                          "gmres_solves": stepper.gmres_calls - counts0[3],
                          "ms_per_gmres_iteration": 1e3 * (stepper.gmres_seconds - counts0[4]) / max(gi, 1),
                          "mean_cfl_used": float(s.cfl * float(used.mean()) / float(dt.mean())),
                          "density_residual": r, "drop": r / r0})
            print(json.dumps(steps[-1]), file=sys.stderr, flush=True)
            if args.bump_log:
                Path(args.bump_log).write_text(json.dumps({"elapsed_s": time.perf_counter() - start,
                                                           "per_step": steps}) + "\n")
            if args.bump_until_drop > 0 and r / r0 <= args.bump_until_drop:
                status = f"density residual fell by {args.bump_until_drop:g} after {k + 1} steps"
                break
    launches = _launches() - before
    vs_oracle = cpu = None
    if args.bump_oracle and first_state is not None:
        from oracle.implicit import ImplicitOracle

        to = time.perf_counter()
        ref, _ = ImplicitOracle(g).step(U0, first_dt, s)
        secs = time.perf_counter() - to
        vs_oracle = {"steps": 1, "state_max_rel_err": max_rel(first_state, ref), "oracle_seconds": secs,
                     "oracle": "oracle/implicit.py: the reference's implicit step over the C residual, SciPy gmres "
                               "and spsolve_triangular, one host thread"}
        cpu = {"value": secs, "unit": "s/step", "cores": 1, "kind": "port",
               "sample": "the first implicit step of the same recipe (oracle restatement, SciPy, one thread)"}
    n = len(steps)
    per_step = sum(x["seconds"] for x in steps) / n if n else None
    estimate = None
    if n and steps[-1]["drop"] < 1.0:
        rate = steps[-1]["drop"] ** (1.0 / n)  # geometric mean drop per step so far
        need = math.log(1e-8) / math.log(rate)
        estimate = {"drop_per_step": rate, "steps_to_8_orders": need, "hours_at_measured_rate": need * per_step / 3600,
                    "basis": f"geometric mean of the first {n} steps"}
    line = {
        "metric": "implicit Euler step, bump channel (s per step)", "value": per_step, "unit": "s/step",
        "n_gpus": 1, "steps": n, "warmup": 0, "higher_is_better": False, "dtype": "f64",
        "data": "synthetic (seeded bump channel, free-stream start)",
        "config": {"workload": f"bump channel {nx}x{ny} ({dg.n_cells} cells), Roe, MUSCL linear, Barth-Jespersen, "
                               f"implicit Euler, local CFL {s.cfl:g}, GMRES({s.gmres_krylov_dimension}) to "
                               f"{s.gmres_tolerance:g} with LU-SGS", "setup_s": setup_s,
                   "budget_s": args.budget_s, "mode": "exact"},
        "status": status, "per_step": steps, "initial_density_residual": r0,
        "ms_per_gmres_iteration": (1e3 * stepper.gmres_seconds / stepper.gmres_iterations
                                   if stepper.gmres_iterations else None),
        "time_to_8_orders": estimate, "vs_oracle": vs_oracle, "cpu_baseline": cpu,
        "gpu_launches": launches, "clocks": clocks.summary(),
    }
    print(json.dumps(line))
    dg.close()


def _launches():
    from meshcfd_gb300._lib import native

    return int(native().mcfd_launch_count())


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch256":
        run_batch(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "bump":
        run_bump(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
