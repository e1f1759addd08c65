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
                    choices=("vortex1024", "vortex1024all", "vortex512", "vortex256", "batch256", "adjoint"))
    ap.add_argument("--checkpoint-every", type=int, default=20)
    ap.add_argument("--batch-adjoint-steps", type=int, default=20)
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--batch-adjoint-checkpoint", type=int, default=5)
    ap.add_argument("--batch-cases", type=int, default=256)
    ap.add_argument("--graph-steps", type=int, default=10)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=10,
                    help="RK3 steps of the CPU baseline sample (about 12 s on one Grace core)")
    ap.add_argument("--profile-steps", type=int, default=3)
    ap.add_argument("--mode", choices=("fast", "exact", "fma"), default="fast",
                    help="exact: reference operation order, bit-exact; fast: exact arithmetic with the "
                         "limiter minimum through the smallest ratio; fma: shared reciprocals + FMA "
                         "(outside the 1e-12 bar on fine meshes)")
    ap.add_argument("--parity-steps", type=int, default=10)
    ap.add_argument("--variant-steps", type=int, default=20)
    return ap.parse_args(argv)


WORKLOADS = {
    "vortex1024": dict(n=1024, split="half"),
    "vortex1024all": dict(n=1024, split="all"),
    "vortex512": dict(n=512, split="half"),
    "vortex256": dict(n=256, split="half"),
}


def _sample_case(name, n):
    """(case, settings, geometry, initial primitive) of workload ``name``,
    at ``n`` x ``n`` quads when given."""
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, vortex_case, vortex_primitive

    w = WORKLOADS[name]
    case, _ = vortex_case(n or w["n"], split=w["split"])
    g = build_geometry(case.mesh, case)
    return case, case.numerics, g, vortex_primitive(cell_centroids(case.mesh))


def make_workload(name):
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.meshes import cell_centroids, vortex_case, vortex_primitive

    w = WORKLOADS[name]
    case, _ = vortex_case(w["n"], split=w["split"])
    settings = case.numerics
    g = build_geometry(case.mesh, case)
    P0 = vortex_primitive(cell_centroids(case.mesh))
    config = {
        "workload": f"isentropic vortex, periodic [0,10]^2, {w['n']}x{w['n']} quads, "
                    f"{'half' if w['split'] == 'half' else 'all'} split to triangles, jitter 0.15h, seed 0",
        "cells": int(len(g.areas)),
        "faces": int(len(g.face_lengths)),
        "interior_faces": int(len(g.interior_faces)),
        "periodic_pairs": int(len(g.periodic_faces_a)),
        "flux": settings.flux, "reconstruction": settings.reconstruction, "limiter": settings.limiter,
        "time_integration": settings.time_integration, "cfl": settings.cfl,
        "time_step_mode": settings.time_step_mode, "precision": "fp64, reference operation order (no FMA)",
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


def cpu_oracle_rate(g, settings, P0, steps):
    """The oracle (C restatement of the reference path, one thread) on the same
    mesh: ``steps`` full RK3 steps including the stable time step."""
    from oracle.oracle import Oracle

    orc = Oracle(g)
    U = orc.conservative(P0, settings.gamma)
    orc.solve(U, settings, 1)  # warm caches / page-in
    t0 = time.perf_counter()
    orc.solve(U, settings, steps)
    dt = time.perf_counter() - t0
    return len(g.areas) * steps / dt, dt


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
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    case, settings, g, P0, config = make_workload(args.workload)
    steps, warm = args.steps, args.warmup
    n = reference_sample(args.workload, steps, warm)
    if n != WORKLOADS[args.workload]["n"]:
        case, settings, g, P0 = _sample_case(args.workload, n)
    from oracle.oracle import Oracle

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
        "config": config,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"{steps} RK3 steps of the same recipe at {n}x{n} quads ({len(g.areas)} "
                                   f"cells{'' if n == WORKLOADS[args.workload]['n'] else ', reduced to fit ~3 min of CPU time'})"
                                   " (oracle: single-threaded C restatement of the reference path; "
                                   "the reference itself is single-threaded NumPy/Numba)"},
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


def run_gpu(args):
    import torch

    from meshcfd_gb300 import _lib
    from meshcfd_gb300.device import DeviceGeometry, make_config

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

    case, settings, g, P0, config = make_workload(args.workload)
    config["parallelism"] = f"replicas x{world}"
    cfg = make_config(settings, mode=args.mode)
    config["precision"] = {
        "exact": "fp64, reference operation order (no FMA), bit-exact",
        "fast": "fp64, reference arithmetic, limiter minimum through the smallest ratio",
        "fma": "fp64, FMA + shared reciprocals",
    }[args.mode]
    native = _lib.native()
    dg = DeviceGeometry(g, device)
    C = dg.n_cells
    from meshcfd_gb300.device import primitive_to_conservative

    U_init = primitive_to_conservative(P0, settings.gamma)
    U = torch.as_tensor(U_init, device=device)
    dt = torch.empty(1, dtype=torch.float64, device=device)
    P = dg.primitive_buffer()
    stream = torch.cuda.current_stream()

    def step():
        dg.time_steps(P, cfg, out_min=dt)
        dg.explicit_step(U, cfg, 2, dt)

    dg.primitive(U, cfg, out=P)
    tuned = dg.autotune(U, cfg) if not args.no_autotune else None
    dg.primitive(U, cfg, out=P)
    for _ in range(args.warmup):
        step()
    dg.check_status()

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    barrier()
    launches0 = native.mcfd_launch_count()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(device.index) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            step()
        stop.record(stream)
        barrier()
    launches = native.mcfd_launch_count() - launches0
    ms, value = replica_throughput(start.elapsed_time(stop), C, args.steps, dist, device)
    dg.check_status()
    ms_per_step = ms / args.steps

    # per-kernel breakdown (CUDA events on the launching stream)
    import ctypes as Cc

    native.mcfd_profile_enable(dg.handle, 1)
    for _ in range(args.profile_steps):
        step()
    tot = (Cc.c_double * 6)()
    grp = (Cc.c_int64 * 6)()
    native.mcfd_profile_read(dg.handle, tot, grp)
    native.mcfd_profile_enable(dg.handle, 0)
    names = ("primitive", "reconstruct", "flux", "gather", "time_step", "other")
    kernels = {names[k]: {"ms_total": tot[k], "groups": int(grp[k]),
                          "ms_per_group": tot[k] / grp[k] if grp[k] else None} for k in range(6) if grp[k]}
    total_ms = sum(v["ms_total"] for v in kernels.values())
    for v in kernels.values():
        v["share"] = v["ms_total"] / total_ms
    mbytes, counts = model_bytes(g)
    dominant = max(kernels, key=lambda k: kernels[k]["ms_total"])
    peak, peak_kind = measured_peaks()
    achieved = mbytes[dominant] / (kernels[dominant]["ms_per_group"] * 1e-3) / 1e9
    traffic = None
    fp64_pipe = alu_pipe = issue = fp64 = None
    tpath = ROOT / "profiles" / "ncu_summary.json"
    if tpath.exists():
        summary = json.loads(tpath.read_text())
        per_cell = summary.get("dram_bytes_per_cell", {}).get(dominant)
        if per_cell:
            traffic = per_cell * C  # ncu capture on the 512^2 mesh of this recipe, scaled by cells
        fp64_pipe = summary.get("fp64_pipe_active_pct", {}).get(dominant)
        alu_pipe = summary.get("alu_pipe_active_pct", {}).get(dominant)
        issue = summary.get("issue_active_pct", {}).get(dominant)
        # the FP64 side of the same kernel: its FP64 instructions per cell
        # (ncu count on the same mesh recipe and mode) over the live launch time
        ipc = summary.get("fp64_instructions_per_cell", {}).get(dominant)
        fpeak = summary.get("fp64_peak_ginstr_s")
        if ipc and fpeak and args.mode == summary.get("mode") and args.workload in ("vortex1024", "vortex512",
                                                                                     "vortex256"):
            got = ipc * C / (kernels[dominant]["ms_per_group"] * 1e-3) / 1e9
            fp64 = {"achieved": got, "peak": fpeak, "unit": "G FP64 thread-instructions/s", "frac": got / fpeak,
                    "instructions_per_cell": ipc,
                    "source": "instructions per cell from the ncu capture of this kernel on the 512^2 mesh of this "
                              "recipe; peak: " + summary.get("fp64_peak_source", "")}
    step_bytes = 3 * (mbytes["reconstruct"] + mbytes["flux"] + mbytes["gather"]) - 32 * C + mbytes["time_step"]
    roofline = {
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
        "note": ("compute bound, not HBM bound: GB300's FP64 pipe issues ~0.5 T instr/s; divisions, square roots "
                 "and part of the products run bit-identically on the integer pipe, and ncu shows the dominant "
                 "kernel sharing the FP64 and ALU pipes (fp64 / alu / issue percentages above); 'fp64' is the "
                 "kernel's FP64 instruction rate against the measured FP64 issue rate"),
    }

    # end to end: state in pinned host memory, H2D + step + D2H every step
    e2e = None
    if not args.no_e2e:
        host = torch.as_tensor(U_init).pin_memory()
        out = torch.empty_like(host).pin_memory()

        def e2e_step():
            U.copy_(host, non_blocking=True)
            dg.primitive(U, cfg, out=P)
            step()
            out.copy_(U, non_blocking=True)

        for _ in range(2):
            e2e_step()
        barrier()
        s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s2.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e2.record(stream)
        barrier()
        ms2 = s2.elapsed_time(e2)
        dg.check_status()
        e2e = {"value": world * C * args.steps / (ms2 * 1e-3), "unit": UNIT,
               "h2d_bytes_per_step": int(host.numel() * 8), "d2h_bytes_per_step": int(out.numel() * 8),
               "ms_per_step": ms2 / args.steps}

    # parity of this run's kernels against the bit-exact path (which the
    # parity tests hold equal to the reference): one residual, and
    # --parity-steps steps, from the initial state of the workload
    parity = None
    if args.parity_steps > 0:
        cfg_exact = make_config(settings, mode="exact")
        U0 = torch.as_tensor(U_init, device=device)
        Ra = dg.residual(U0, cfg)
        Rb = dg.residual(U0, cfg_exact)
        res_err = float((Ra - Rb).abs().max() / Rb.abs().max())
        Ua, Ub = U0.clone(), U0.clone()
        for Uc, cf in ((Ua, cfg), (Ub, cfg_exact)):
            Pc = dg.primitive(Uc, cf)
            Pc = Pc.clone()
            for _ in range(args.parity_steps):
                dg.time_steps(Pc, cf, out_min=dt)
                dg.explicit_step(Uc, cf, 2, dt)
                Pc = dg.primitive(Uc, cf)
        dg.check_status()
        parity = {"reference": "bit-exact path (equal to the reference, see tests/test_gpu_parity.py)",
                  "residual_max_rel_err": res_err, "steps": args.parity_steps,
                  "state_max_rel_err": float((Ua - Ub).abs().max() / Ub.abs().max())}

    # the other kernel variants on the same workload: step time and the
    # residual's deviation from the bit-exact path
    variants = {}
    if args.variant_steps > 0:
        cfg_exact = make_config(settings, mode="exact")
        U0 = torch.as_tensor(U_init, device=device)
        Rb = dg.residual(U0, cfg_exact)
        for mode in ("exact", "fast", "fma"):
            cf = make_config(settings, mode=mode)
            Ra = dg.residual(U0, cf)
            err = float((Ra - Rb).abs().max() / Rb.abs().max())
            Uv = U0.clone()
            dg.primitive(Uv, cf, out=P)
            for _ in range(2):
                dg.time_steps(P, cf, out_min=dt)
                dg.explicit_step(Uv, cf, 2, dt)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(args.variant_steps):
                dg.time_steps(P, cf, out_min=dt)
                dg.explicit_step(Uv, cf, 2, dt)
            b.record(stream)
            torch.cuda.synchronize()
            msv = a.elapsed_time(b) / args.variant_steps
            variants[mode] = {"ms_per_step": msv, "value": C / (msv * 1e-3), "residual_max_rel_err": err}
        dg.check_status()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, secs = cpu_oracle_rate(g, settings, P0, args.cpu_steps)
        cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{args.cpu_steps} RK3 steps of the same {C}-cell workload in {secs:.1f} s "
                         "(oracle: single-threaded C restatement of the reference path)"}
    clock = clocks.summary()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded vortex mesh and state)",
            "config": config, "gpu_launches": int(launches), "roofline": roofline, "kernels": kernels,
            "autotune": tuned,
            "e2e": e2e, "cpu_baseline": cpu, "clocks": clock, "parity": parity, "mode": args.mode,
            "variants": variants,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def run_batch(args):
    """Batching workload: the seeded 256 uneven channel/Riemann cases (HLLC,
    MUSCL-Venkatakrishnan, RK3), all cases in one geometry with one launch per
    kernel per stage, steps captured in a CUDA graph, against the same cases
    solved one at a time with the plain path (host loop per case)."""
    import torch

    from meshcfd_gb300.batch import BatchStepper, batch_workload, build_batch
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.solver import run_explicit
    from meshcfd_gb300.device import primitive_to_conservative

    device = torch.device("cuda", 0)
    t0 = time.perf_counter()
    cases = batch_workload(n_cases=args.batch_cases)
    geo, layout, P0, geoms = build_batch(cases)
    settings = cases[0][0].numerics
    U0 = primitive_to_conservative(P0, settings.gamma)
    dg = DeviceGeometry(geo, device)
    setup_s = time.perf_counter() - t0
    steps = args.steps
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
    with ClockSampler(0) as clocks:
        a.record()
        for _ in range(reps):
            stepper.replay()
        b.record()
        torch.cuda.synchronize()
    dg.check_status()
    batched_ms = a.elapsed_time(b)
    done_steps = reps * gsteps
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
    n_cells = int(dg.n_cells)
    value = layout.n_cases * done_steps / (batched_ms * 1e-3)
    adjoint = None
    if args.batch_adjoint_steps > 0:
        adjoint = batched_adjoint(dg, layout, settings, U0, stepper, args)
    line = {
        "metric": "batched case-steps/s (RK3 HLLC-MUSCL, 256 uneven cases)", "value": value, "unit": "case-steps/s",
        "n_gpus": 1, "steps": done_steps, "warmup": args.warmup, "ms_per_step": batched_ms / done_steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded channel/Riemann cases)",
        "config": {"workload": f"{layout.n_cases} channel/Riemann cases, cells log-uniform [2k,200k], aspect U[1,4], "
                               f"Mach U[0.3,2.0], seed 3", "cells_total": n_cells, "mode": args.mode,
                   "graph_steps": gsteps, "setup_s": setup_s},
        "batched": {"cell_updates_per_s": n_cells * done_steps / (batched_ms * 1e-3), "ms": batched_ms},
        "one_at_a_time": {"case_steps_per_s": layout.n_cases * done_steps / (single_ms * 1e-3), "ms": single_ms},
        "batched_over_one_at_a_time": single_ms / batched_ms,
        "bit_identical": bool(same), "clocks": clocks.summary(),
        "batched_adjoint": adjoint, "autotune": tuned,
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


def run_adjoint(args):
    """Adjoint workload: O-grid 1024x512 around a cylinder (seed 2, Mach 0.3
    free stream, slip wall, far field), HLLC / MUSCL-Venkatakrishnan, RK3 with
    a fixed time step for ``--steps`` steps (default 400 here), checkpoints
    every ``--checkpoint-every`` steps; the wall pressure force along x at the
    final state and its gradient with respect to the initial state and the
    far-field states by the discrete adjoint.  Reports the adjoint / forward
    cost ratio (lower is better)."""
    import torch

    from meshcfd_gb300.adjoint import WallForceAdjoint
    from meshcfd_gb300.device import DeviceGeometry
    from meshcfd_gb300.geometry import build_geometry
    from meshcfd_gb300.device import make_config, primitive_to_conservative
    from meshcfd_gb300.meshes import ogrid_case

    device = torch.device("cuda", 0)
    steps = args.steps if args.steps != 100 else 400
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
    with ClockSampler(0) as clocks:
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
    line = {
        "metric": "RK3 wall-force adjoint / forward cost ratio", "value": adj_ms / fwd_ms, "unit": "ratio",
        "n_gpus": 1, "steps": steps, "warmup": args.warmup, "ms_per_step": (fwd_ms + adj_ms) / steps,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded O-grid, free-stream start)",
        "config": {"workload": f"O-grid 1024x512 around a cylinder ({C} cells), Mach 0.3, HLLC, MUSCL linear, "
                               f"Venkatakrishnan, RK3 fixed dt, {steps} steps, checkpoint every "
                               f"{args.checkpoint_every}", "mode": args.mode, "dt": dt, "setup_s": setup_s,
                   "l2_flush": "working set larger than L2"},
        "forward": {"ms": fwd_ms, "cell_updates_per_s": C * steps / (fwd_ms * 1e-3)},
        "adjoint": {"ms": adj_ms, "cell_updates_per_s": C * steps / (adj_ms * 1e-3),
                    "work_per_step": "1 replayed RK3 step + 3 residual VJPs"},
        "J": J, "grad_norm": float(lam0.norm()), "far_grad_norm": float(adj.far_acc.norm()),
        "gpu_launches": launches, "clocks": clocks.summary(),
    }
    print(json.dumps(line))


def _launches():
    from meshcfd_gb300._lib import native

    return int(native().mcfd_launch_count())


def main():
    args = parse()
    if args.workload == "batch256":
        run_batch(args)
        return
    if args.workload == "adjoint":
        run_adjoint(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
