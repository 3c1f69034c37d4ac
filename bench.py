"""Benchmark of the steady Euler residual/update path on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]
                    [--workload explicit_bump_72k]

Default workload: implicit backward Euler on the 200x60x30-hex bump channel (2.16M tets,
Mach 0.84), block-ILU(0) GMRES(30) to 1e-2, CFL ramp 10 -> 1000 over 50 steps; the line's value
is the FP32-system defect correction (FP64 residual and update), with the plain FP64 system
measured on the same steps beside it.  A step is one pseudo-time step (explicit workloads: one
4-stage iteration) over every cell; the metric is cell-updates/s = cells x steps / time.  Rank 0
prints one JSON line.

* value: device time from CUDA events on the library's stream around each step's graph
  launch, L2 flushed (256 MB write) before every timed step, summed over K steps; max over
  ranks.
* e2e: the same steps through the C ABI with host buffers: every step uploads the state,
  runs one iteration (bes_explicit_iterations, which reads the residual norms back) and
  downloads the state; wall clock.
* roofline: the dominant kernel's algorithmic bytes per launch / its average event-timed
  launch duration, against the measured HBM copy bandwidth.
* cpu_baseline: the CPU restatement of the reference (OpenMP, all host cores) on a bounded
  sample of the same workload (rank 0 only).
N > 1 runs independent replicas (the path has no collective): weak scaling.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s"
METRIC_FULL = ("converged solves/hour at 1e-8 residual drop vs plain FP64 GPU; cell-updates/s")

WORKLOADS = {
    # explicit FP64, 60x20x10-hex bump channel (72,000 tets), Mach 0.5, local dt at CFL 0.8
    "explicit_bump_72k": dict(kind="explicit", mesh=("bump", 60, 20, 10, 0.04),
                              opts=dict(solver_type=0, local_time_step=1, courant_num=0.8,
                                        freestream_mach=(0.5, 0.0, 0.0))),
    # 120x40x18-hex channel (518,400 tets): a profiling size whose working set exceeds L2
    "explicit_bump_518k": dict(kind="explicit", mesh=("bump", 120, 40, 18, 0.08),
                               opts=dict(solver_type=0, local_time_step=1, courant_num=0.8,
                                         freestream_mach=(0.84, 0.0, 0.0))),
    # implicit backward Euler on the 200x60x30-hex channel (2.16M tets), bump 0.08, Mach 0.84:
    # first-order Roe Jacobian in 5x5 blocks, block-ILU(0) GMRES(30) to 1e-2 relative, CFL
    # ramped 10 -> 1000 over 50 steps; FP32 Jacobian/preconditioner/Krylov with FP64 residual
    # and update (defect correction), or everything FP64
    "implicit_bump_2m": dict(kind="implicit", mesh=("bump", 200, 60, 30, 0.08), converge=300,
                                   opts=dict(solver_type=1, local_time_step=1, courant_num=10.0,
                                             freestream_mach=(0.84, 0.0, 0.0), linear_solver=1,
                                             linear_solver_tol=1e-2, linear_solver_max_iter=300,
                                             gmres_restart=30, cfl_ramp_steps=50,
                                             cfl_ramp_start=10.0, cfl_ramp_end=1000.0,
                                             precision=2)),
    # the same with the FP32 system stored in FP32 (precision 1)
    "implicit_bump_2m_fp32": dict(kind="implicit", mesh=("bump", 200, 60, 30, 0.08),
                                  opts=dict(solver_type=1, local_time_step=1, courant_num=10.0,
                                            freestream_mach=(0.84, 0.0, 0.0), linear_solver=1,
                                            linear_solver_tol=1e-2, linear_solver_max_iter=300,
                                            gmres_restart=30, cfl_ramp_steps=50,
                                            cfl_ramp_start=10.0, cfl_ramp_end=1000.0,
                                            precision=1)),
    # the same scheme on the 60x20x10-hex channel (72,000 tets): the CPU-runnable size
    "implicit_bump_72k": dict(kind="implicit", mesh=("bump", 60, 20, 10, 0.08),
                              opts=dict(solver_type=1, local_time_step=1, courant_num=10.0,
                                        freestream_mach=(0.84, 0.0, 0.0), linear_solver=1,
                                        linear_solver_tol=1e-2, linear_solver_max_iter=300,
                                        gmres_restart=30, cfl_ramp_steps=50,
                                        cfl_ramp_start=10.0, cfl_ramp_end=1000.0,
                                        precision=2)),
    # the same scheme on the 120x40x18-hex channel (518,400 tets): a profiling size whose
    # Krylov basis (31 vectors of 10 MB) still exceeds L2
    "implicit_bump_518k": dict(kind="implicit", mesh=("bump", 120, 40, 18, 0.08),
                               opts=dict(solver_type=1, local_time_step=1, courant_num=10.0,
                                         freestream_mach=(0.84, 0.0, 0.0), linear_solver=1,
                                         linear_solver_tol=1e-2, linear_solver_max_iter=300,
                                         gmres_restart=30, cfl_ramp_steps=50,
                                         cfl_ramp_start=10.0, cfl_ramp_end=1000.0,
                                         precision=2)),
    "implicit_bump_2m_fp64": dict(kind="implicit", mesh=("bump", 200, 60, 30, 0.08),
                                  opts=dict(solver_type=1, local_time_step=1, courant_num=10.0,
                                            freestream_mach=(0.84, 0.0, 0.0), linear_solver=1,
                                            linear_solver_tol=1e-2, linear_solver_max_iter=300,
                                            gmres_restart=30, cfl_ramp_steps=50,
                                            cfl_ramp_start=10.0, cfl_ramp_end=1000.0,
                                            precision=0)),
    # batched sweep: 64 freestream conditions (numpy seed 0: Mach 0.3-0.85, pitch and sideslip
    # -4..4 deg) on the 100x50x100-hex Gaussian-bump box (3.0M tets, stretching 1.05), explicit
    # local dt at CFL 0.8, all conditions advanced by one graph launch per iteration
    "sweep_gauss_3m_64": dict(kind="explicit", mesh=("gauss", 100, 50, 100, 1.05),
                              conds=(0, 64),
                              opts=dict(solver_type=0, local_time_step=1, courant_num=0.8)),
    # learned warm start with the explicit solver: 30x15x30-hex Gaussian
    # box (81,000 tets); training data = the batched explicit solver's states after 1500
    # iterations for 32 conditions (seed 1); 8 held-out conditions (seed 2) run from the
    # network's prediction and from the freestream
    "warmstart_gauss_81k": dict(kind="warmstart", mesh=("gauss", 30, 15, 30, 1.05),
                                train=(1, 32), test=(2, 8), data_iters=1500, eval_iters=1500,
                                train_steps=3000, batch=8192,
                                opts=dict(solver_type=0, local_time_step=1, courant_num=0.8)),
    # learned warm start at full size: the Gaussian-bump box at 60x30x60
    # hexes (648,000 tets); training data = 512 conditions (seed 1) solved to a 1e-8 drop by the
    # batched implicit sweep (FP32 system with 16-bit storage, linear tolerance prod_tol); the
    # network trained for 20,000 AdamW steps (lr 1e-3) on the converged ones; 64 held-out
    # conditions (seed 2) solved from its prediction and from the freestream to the same
    # absolute residual (1e-8 x the freestream state's residual), and the plain FP64 solver on
    # the first plain_sample of them for the reference answer
    "production_gauss_648k": dict(kind="production", mesh=("gauss", 60, 30, 60, 1.05),
                                  train=(1, 512), test=(2, 64), plain_sample=4, slots=32,
                                  data_max_steps=150, data_budget_s=1200.0, max_steps=200,
                                  train_steps=20000,
                                  batch=8192, prod_tol=0.1,
                                  opts=dict(solver_type=1, local_time_step=1, courant_num=10.0,
                                            linear_solver=1, linear_solver_tol=1e-2,
                                            linear_solver_max_iter=300, gmres_restart=30,
                                            cfl_ramp_steps=50, cfl_ramp_start=10.0,
                                            cfl_ramp_end=1000.0, precision=2)),
    # the same scheme at a validation size (30x15x30 hexes, 81,000 tets; 32 training and 8
    # held-out conditions, 3,000 AdamW steps)
    "production_gauss_81k": dict(kind="production", mesh=("gauss", 30, 15, 30, 1.05),
                                 train=(1, 32), test=(2, 8), plain_sample=2, slots=8,
                                 data_max_steps=200, max_steps=300, train_steps=3000,
                                 batch=8192, prod_tol=0.1,
                                 opts=dict(solver_type=1, local_time_step=1, courant_num=10.0,
                                           linear_solver=1, linear_solver_tol=1e-2,
                                           linear_solver_max_iter=300, gmres_restart=30,
                                           cfl_ramp_steps=50, cfl_ramp_start=10.0,
                                           cfl_ramp_end=1000.0, precision=2)),
    # production form at scale: the Gaussian-bump box at 200x100x200 hexes (24.0M tets), the
    # 16 conditions of seed 3, as many of them as one GB300's memory holds as slots of one
    # batched implicit context (precision 2, the benchmark's GMRES settings); a throughput
    # measurement of whole batched steps, not converged solves
    "implicit_gauss_24m_16": dict(kind="scale", mesh=("gauss", 200, 100, 200, 1.05), conds=(3, 16),
                                  opts=dict(solver_type=1, local_time_step=1, courant_num=10.0,
                                            linear_solver=1, linear_solver_tol=1e-2,
                                            linear_solver_max_iter=300, gmres_restart=30,
                                            cfl_ramp_steps=50, cfl_ramp_start=10.0,
                                            cfl_ramp_end=1000.0, precision=2)),
    # converged batched sweep: 64 freestream conditions (numpy seed 0: Mach 0.3-0.85, pitch and
    # sideslip -4..4 deg) on the 100x50x100-hex Gaussian-bump box (3.0M tets, stretching 1.05),
    # each solved to a 1e-8 drop of its residual L2.  Production form: FP32 system with 16-bit
    # block storage and FP64 residual/update, all conditions through the slots of one batched
    # context (one graph launch per step of every slot, a converged slot takes the next
    # condition), linear solves to prod_tol; plain form: the FP64 system, one condition per
    # context, linear solves to 1e-2, on the first `plain_sample` conditions
    "sweep_implicit_gauss_3m_64": dict(kind="isweep", mesh=("gauss", 100, 50, 100, 1.05),
                                       conds=(0, 64), plain_sample=4, max_steps=300, slots=32,
                                       prod_tol=0.1,
                                       opts=dict(solver_type=1, local_time_step=1,
                                                 courant_num=10.0, linear_solver=1,
                                                 linear_solver_tol=1e-2,
                                                 linear_solver_max_iter=300, gmres_restart=30,
                                                 cfl_ramp_steps=50, cfl_ramp_start=10.0,
                                                 cfl_ramp_end=1000.0, precision=2)),
    # the same sweep at a validation size: 30x15x30-hex box (81,000 tets), 8 conditions
    "sweep_implicit_gauss_81k_8": dict(kind="isweep", mesh=("gauss", 30, 15, 30, 1.05),
                                       conds=(0, 8), plain_sample=2, max_steps=400, slots=4,
                                       prod_tol=0.1,
                                       opts=dict(solver_type=1, local_time_step=1,
                                                 courant_num=10.0, linear_solver=1,
                                                 linear_solver_tol=1e-2,
                                                 linear_solver_max_iter=300, gmres_restart=30,
                                                 cfl_ramp_steps=50, cfl_ramp_start=10.0,
                                                 cfl_ramp_end=1000.0, precision=2)),
    # same scheme on the 200x60x30-hex channel (2.16M tets), Mach 0.84
    "explicit_bump_2m": dict(kind="explicit", mesh=("bump", 200, 60, 30, 0.08),
                             opts=dict(solver_type=0, local_time_step=1, courant_num=0.8,
                                       freestream_mach=(0.84, 0.0, 0.0))),
}

# bytes each kernel must move per unit (compulsory traffic of the SoA layout, FP64):
#   cell sweep per cell: state of the cell (40) + Sc (96) + w (32) + r (96) + adj (16)
#     + flags (1) + 1/V (8) + eps^2 (8) + face-side state written (40)      = 337
#     (stage 0 adds plen 24 + V 8 + dt 8 = 40; neighbour states are re-reads of the same array)
#   face flux per face: RS indices (8) + normal (24) + area (8) + two side states (80)
#     + flux x area written (40)                                            = 160
#   update per cell: 4 face ids (16) + 4 fluxes (160) + U(n) (40) + dt (8) + 1/V (8)
#     + U written (40)                                                      = 272
BYTES_PER_CELL_SWEEP = 337.0
BYTES_PER_FACE = 160.0
BYTES_PER_UPDATE = 272.0


def make_mesh(spec):
    from bes_gb300 import meshgen
    if spec[0] == "bump":
        return meshgen.bump_channel(*spec[1:])
    return meshgen.gaussian_box(*spec[1:])


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(x: float, dist) -> float:
    """The largest value of x over the ranks of the process group (x itself on one rank)."""
    if not dist:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profiles(kernel: str, workload: str, precision: int = 1):
    """Per-launch DRAM bytes of `kernel` (at `precision` for the implicit system) from a
    committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    key = f"{kernel}_packed" if precision == 2 else kernel
    return d.get(workload, {}).get(key)


def cpu_baseline(wl, mesh, steps: int = 2, mach=None):
    """The CPU restatement (reference operation order, OpenMP on all host cores), one
    condition."""
    from oracle import pyoracle
    o = wl["opts"]
    threads = os.cpu_count() or 1
    mach = o["freestream_mach"] if mach is None else tuple(mach)
    O = pyoracle.Oracle(mesh, cfl=o["courant_num"], mach=mach,
                        local_dt=o["local_time_step"], threads=threads)
    O.explicit_run(1)  # warm-up
    t0 = time.perf_counter()
    O.explicit_run(steps)
    dt = time.perf_counter() - t0
    return {"value": mesh.n_cells * steps / dt, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{steps} explicit iterations on the full {mesh.n_cells}-cell mesh "
                      f"(oracle/bes_oracle.cpp, OpenMP {threads} threads)"}


def run_reference(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    if wl["kind"] == "implicit":
        # the same mesh and options as the GPU arm; whole implicit steps from the freestream,
        # as many as fit in about two minutes (the GPU arm times steps warmup+1..warmup+steps)
        mesh = make_mesh(wl["mesh"])
        base = implicit_cpu_baseline(wl, mesh, max_seconds=120.0, max_steps=args.steps)
        value = base["value"]
        line = {"impl": "reference", "metric": METRIC, "metric_full": METRIC_FULL,
                "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": base["steps"],
                "warmup": 0, "ms_per_step": base["seconds"] / base["steps"] * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic",
                "config": {"workload": args.workload, "cells": mesh.n_cells,
                           "timed_steps": f"1-{base['steps']} from the freestream",
                           "linear_iterations_per_step": base["linear_iterations_per_step"]},
                "cpu_baseline": base,
                "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0
    if wl["kind"] in ("production", "scale", "isweep"):
        # one condition of the sweep on the same mesh, whole implicit steps from the freestream
        from bes_gb300 import meshgen
        mesh = make_mesh(wl["mesh"])
        seed, n = wl["conds"] if "conds" in wl else wl["train"]
        mach = meshgen.freestream_mach_vector(*meshgen.sample_conditions(n, seed)[0])
        wl1 = dict(wl, opts=dict(wl["opts"], freestream_mach=tuple(mach)))
        base = implicit_cpu_baseline(wl1, mesh, max_seconds=120.0, max_steps=args.steps)
        value = base["value"]
        line = {"impl": "reference", "metric": METRIC, "metric_full": METRIC_FULL,
                "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": base["steps"],
                "warmup": 0, "ms_per_step": base["seconds"] / base["steps"] * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic",
                "config": {"workload": args.workload, "cells": mesh.n_cells,
                           "timed_steps": f"1-{base['steps']} of the first condition"},
                "cpu_baseline": base,
                "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0
    mesh = make_mesh(wl["mesh"])
    steps = args.steps
    from oracle import pyoracle
    o = wl["opts"]
    threads = os.cpu_count() or 1
    mach = o.get("freestream_mach")
    if mach is None:  # a sweep: the reference runs one condition per process, time the first
        from bes_gb300 import meshgen
        seed, n = wl["conds"] if "conds" in wl else wl["train"]
        mach = meshgen.freestream_mach_vector(*meshgen.sample_conditions(n, seed)[0])
    O = pyoracle.Oracle(mesh, cfl=o["courant_num"], mach=mach,
                        local_dt=o["local_time_step"], threads=threads)
    O.explicit_run(max(1, min(args.warmup, 2)))
    # each step: one full explicit iteration on the whole mesh; bounded to about 3 minutes
    t0 = time.perf_counter()
    done = 0
    for _ in range(steps):
        O.explicit_run(1)
        done += 1
        if time.perf_counter() - t0 > 180:
            break
    dt = time.perf_counter() - t0
    value = mesh.n_cells * done / dt
    line = {"impl": "reference", "metric": METRIC, "metric_full": METRIC_FULL, "value": value,
            "unit": METRIC, "n_gpus": args.gpus, "steps": done, "warmup": args.warmup,
            "ms_per_step": dt / done * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "cells": mesh.n_cells},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": f"{done} explicit iterations on the full mesh; the "
                                       "reference's CPU path restated in oracle/ (the reference "
                                       "sources are not available on this host)"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# Algorithmic bytes per cell of the implicit kernels with an FP32 system (4-byte values):
#   preconditioner application (colour-ordered block ILU(0) forward + backward sweep): the
#     four off-diagonal blocks once (4 x 100) + inverse diagonal block (100) + the vector read
#     and written in both sweeps (4 x 20)                                          = 580
#   matrix-vector product: five blocks (500) + x (20) + y (20)                       = 540
# With an FP64 system the block and vector bytes double.  With 16-bit block-scaled storage
# (precision 2) a block is 13 half2 words + one FP32 scale = 56 bytes: preconditioner
# 5 x 56 + 80 = 360, matrix-vector product 5 x 56 + 40 = 320.
BYTES_PRECOND = {2: 360.0, 1: 580.0, 0: 1160.0}
BYTES_SPMV = {2: 320.0, 1: 540.0, 0: 1080.0}
KERNEL_NAMES = {
    "precond": {2: "block-ILU(0) colour sweeps, packed blocks (ilu_colour_packed_kernel)",
                1: "block-ILU(0) colour sweeps (ilu_colour_kernel)",
                0: "block-ILU(0) colour sweeps (ilu_colour_kernel)"},
    "spmv": {2: "spmv_packed_kernel", 1: "spmv_kernel", 0: "spmv_kernel"}}


# FP64 floating-point operations per unit of the explicit path, counted: the fluxes by
# instantiating the GPU's flux templates on a counting scalar (tests/opcount), the cell sweep
# and the update per loop from their source (add, sub and mul count 1 each; the divisions and
# square roots, 5 per cell and stage and 4 + 3 per face, come on top)
FLOPS_PER_CELL_STAGE = 646  # cell sweep 614 (gradient 184, 1/V 15, limiter 370, MUSCL 45), update 32
FLOPS_PER_CELL_DT = 33      # local time step, once per iteration
FLOPS_PER_UPDATE = 32       # update kernel per cell and stage (part of FLOPS_PER_CELL_STAGE)
FLOPS_PER_FACE_STAGE = 186  # Roe flux 181 + flux x area 5 (boundary faces need fewer)


def explicit_fp64_work(nc: int, nf: int, cell_updates_per_s: float, n_stage: int = 4) -> dict:
    """Counted FP64 work of one explicit iteration per cell and the rate it was done at."""
    per_iter = (nc * (n_stage * FLOPS_PER_CELL_STAGE + FLOPS_PER_CELL_DT)
                + nf * n_stage * FLOPS_PER_FACE_STAGE)
    per_cell = per_iter / nc
    return {"flops_per_cell_update": per_cell,
            "achieved_tflops": cell_updates_per_s * per_cell / 1e12,
            "note": "add/sub/mul counted once each (divisions and square roots on top); the "
                    "cell sweep and the face flux are FP64-issue bound on this GPU"}


def implicit_leg(args, torch, ctx, steps, warmup, flush, with_e2e, prof_steps: int = 5):
    """warm-up, then `steps` timed implicit steps (events on the library stream around each
    step's graph launch, L2 flushed before each); then `prof_steps` more steps with the step
    graph's device timer stamps on, for the kernel-category profile (the stamps are kernels of
    their own, kept out of the timed steps).  Returns timing, history, state and profile."""
    ctx.implicit_steps(warmup)
    ext = torch.cuda.ExternalStream(ctx.stream_handle)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    c0 = ctx.counters()
    s0 = ctx.implicit_stats()
    hist = []
    torch.cuda.synchronize()
    for k in range(steps):
        with torch.cuda.stream(ext):
            flush.fill_(float(k))
            starts[k].record(ext)
        hist.append(ctx.implicit_steps(1)[0])
        ends[k].record(ext)
    torch.cuda.synchronize()
    c1 = ctx.counters()
    s1 = ctx.implicit_stats()
    dev_ms = float(sum(a.elapsed_time(b) for a, b in zip(starts, ends)))
    out = dict(ms=dev_ms, hist=np.array(hist),
               launches=c1["launches"] - c0["launches"], state=ctx.get_state(),
               force=ctx.wall_force(),
               host_syncs_per_step=(s1["host_syncs"] - s0["host_syncs"]) / steps,
               restart_cycles_per_step=(s1["restart_cycles"] - s0["restart_cycles"]) / steps)
    if prof_steps > 0:
        ctx.profile(True)
        ph = ctx.implicit_steps(prof_steps)
        out["prof"] = ctx.profile(False)
        out["prof_steps"] = prof_steps
        out["prof_linear_iterations"] = float(ph[..., 12].sum())
    if with_e2e:
        U = ctx.get_state()
        t0 = time.perf_counter()
        for _ in range(steps):
            ctx.set_state(U)
            ctx.implicit_steps(1)
            U = ctx.get_state()
        out["e2e_s"] = time.perf_counter() - t0
    return out


def implicit_cpu_baseline(wl, mesh, max_seconds: float = 45.0, max_steps: int = 20):
    """The CPU restatement of the reference's implicit path on the SAME mesh and options as the
    GPU arm (OpenMP on all host cores for the residual and Jacobian assembly; the block-ILU(0)
    GMRES solve is serial, in the reference's file order), timed from the freestream over as
    many whole steps as fit in `max_seconds` (at least one)."""
    from oracle import pyoracle
    o = wl["opts"]
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    O = pyoracle.Oracle(mesh, solver=1, local_dt=o["local_time_step"], cfl=o["courant_num"],
                        mach=o.get("freestream_mach", (0.84, 0.0, 0.0)), lin_precond=1,
                        lin_tol=o["linear_solver_tol"], lin_maxiter=o["linear_solver_max_iter"],
                        lin_restart=o["gmres_restart"], ramp_steps=o["cfl_ramp_steps"],
                        ramp_cfl0=o["cfl_ramp_start"], ramp_cfl1=o["cfl_ramp_end"],
                        threads=threads)
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    done, lin = 0, 0
    while done < max_steps:
        h = O.implicit_run(1)
        done += 1
        lin += int(h[0, 12])
        if time.perf_counter() - t0 > max_seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": mesh.n_cells * done / dt, "unit": METRIC, "cores": threads, "kind": "port",
            "steps": done, "seconds": dt, "setup_seconds": t_setup,
            "linear_iterations_per_step": lin / done,
            "sample": f"implicit steps 1-{done} from the freestream (block-ILU(0) GMRES, FP64) "
                      f"on the same {mesh.n_cells}-cell mesh and options as the GPU arm "
                      f"(oracle/bes_oracle.cpp; OpenMP {threads} threads in the residual and "
                      f"Jacobian assembly, serial linear solve)"}


def run_implicit(args, wl, torch, ctx, mesh, world, rank, local_rank, dist):
    """One step = one implicit pseudo-time step (residual, Jacobian, assembly, linear solve,
    update).  value: the FP32-system defect correction (production form); the plain FP64
    system is measured on the same steps for comparison."""
    from bes_gb300 import lib
    nc = ctx.n_cells
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    clocks.start()
    mixed = implicit_leg(args, torch, ctx, args.steps, args.warmup, flush, with_e2e=False)
    clk = clocks.stop()
    t_max = max_over_ranks(mixed["ms"], dist)
    value = world * nc * args.steps / (t_max / 1e3)
    # e2e through the C ABI with host buffers (state up, one step, state down), on the same
    # steps: the solve restarts from the freestream and replays the warm-up untimed
    ctx.set_freestream_state()
    ctx.implicit_steps(args.warmup)
    U = ctx.get_state()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.set_state(U)
        ctx.implicit_steps(1)
        U = ctx.get_state()
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, dist)
    # the plain FP64 system on the same steps
    o64 = dict(wl["opts"])
    o64["precision"] = 0
    ctx64 = lib.Context(mesh, lib.default_options(**o64))
    plain = implicit_leg(args, torch, ctx64, args.steps, args.warmup, flush, with_e2e=False,
                         prof_steps=0)
    ctx64.close()
    prec = int(wl["opts"].get("precision", 0))
    fp32 = None
    if prec == 2:
        # the FP32 system stored in FP32 (precision 1) on the same steps
        c32 = lib.Context(mesh, lib.default_options(**dict(wl["opts"], precision=1)))
        fp32 = implicit_leg(args, torch, c32, args.steps, args.warmup, flush, with_e2e=False,
                            prof_steps=0)
        c32.close()
    prof = mixed["prof"]
    cats = {"precond": BYTES_PRECOND[prec] * nc, "spmv": BYTES_SPMV[prec] * nc}
    dom = max(cats, key=lambda k: prof[k][0])
    per_launch_ms = prof[dom][0] / max(prof[dom][1], 1)
    achieved = cats[dom] / (per_launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    hist = mixed["hist"]
    line = {"metric": METRIC, "metric_full": METRIC_FULL, "value": value, "unit": METRIC,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": {0: "f64", 1: "f32 system / f64 residual and update",
                      2: "f32 system stored as fp16 blocks with a power-of-two scale per block "
                         "/ f64 residual and update"}[prec],
            "data": "synthetic",
            "config": {"workload": args.workload, "cells": nc, "faces": ctx.n_faces,
                       "parallelism": f"replicas{world}",
                       "l2": "flushed before every timed step (256 MB write)",
                       "linear_iterations_per_step": float(hist[:, 12].mean()),
                       "cfl_range": [float(hist[0, 10]), float(hist[-1, 10])]},
            "fp64_plain": {"value": world * nc * args.steps / (plain["ms"] / 1e3),
                           "ms_per_step": plain["ms"] / args.steps,
                           "linear_iterations_per_step": float(plain["hist"][:, 12].mean()),
                           "mixed_over_fp64": plain["ms"] / mixed["ms"]},
            # the FP32-system run against the FP64-system run after the same steps
            "error_vs_fp64": {
                "state_rel_l2": float(np.linalg.norm(mixed["state"] - plain["state"])
                                      / np.linalg.norm(plain["state"])),
                "force_rel": float(np.linalg.norm(mixed["force"] - plain["force"])
                                   / np.linalg.norm(plain["force"]))},
            "e2e": {"value": world * nc * args.steps / e2e_s, "unit": METRIC,
                    "h2d_bytes_per_step": 40 * nc, "d2h_bytes_per_step": 40 * nc},
            "gpu_launches": mixed["launches"],
            "host_syncs_per_step": mixed["host_syncs_per_step"],
            "tuning": ctx.tuning().strip(),
            "restart_cycles_per_step": mixed["restart_cycles_per_step"],
            "roofline": {"kernel": KERNEL_NAMES[dom][prec],
                         "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": traffic_from_profiles(dom, args.workload, prec),
                         "ms_per_launch": per_launch_ms, "bytes_per_launch": cats[dom],
                         "timing": f"device timer stamps around each launch group inside the "
                                   f"step graph, {mixed['prof_steps']} steps after the timed ones",
                         "category_ms_per_step": {k: v[0] / mixed["prof_steps"]
                                                  for k, v in prof.items()}},
            "clocks": clk}
    if fp32 is not None:
        line["fp32_storage"] = {"value": world * nc * args.steps / (fp32["ms"] / 1e3),
                                "ms_per_step": fp32["ms"] / args.steps,
                                "linear_iterations_per_step": float(fp32["hist"][:, 12].mean()),
                                "state_rel_l2_vs_fp64": float(
                                    np.linalg.norm(fp32["state"] - plain["state"])
                                    / np.linalg.norm(plain["state"]))}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = implicit_cpu_baseline(wl, mesh)
        line["error_vs_fp64_oracle"] = oracle_error(wl, mesh, lib)
    return line


def oracle_error(wl, mesh, lib, steps: int = 2):
    """The GPU's FP64 system and the production form against the FP64 oracle (the CPU
    restatement given the GPU's block-ILU(0) order) over the first `steps` implicit steps
    from the freestream on the workload's own mesh."""
    from oracle import pyoracle
    o = wl["opts"]
    out = {"steps": steps}
    states = {}
    for name, prec in (("fp64_system", 0), ("production", int(o.get("precision", 0)))):
        c = lib.Context(mesh, lib.default_options(**dict(o, precision=prec)))
        h = c.implicit_steps(steps)
        states[name] = (c.get_state(), h)
        order = c.ilu_order()
        c.close()
    O = pyoracle.Oracle(mesh, solver=1, local_dt=o["local_time_step"], cfl=o["courant_num"],
                        mach=o.get("freestream_mach", (0.84, 0.0, 0.0)), lin_precond=1,
                        lin_tol=o["linear_solver_tol"], lin_maxiter=o["linear_solver_max_iter"],
                        lin_restart=o["gmres_restart"], ramp_steps=o["cfl_ramp_steps"],
                        ramp_cfl0=o["cfl_ramp_start"], ramp_cfl1=o["cfl_ramp_end"],
                        threads=os.cpu_count() or 1)
    O.set_ilu_order(order)
    ho = O.implicit_run(steps)
    Uo = O.get_state()
    for name, (U, h) in states.items():
        out[name] = {"state_rel_l2": float(np.linalg.norm(U - Uo) / np.linalg.norm(Uo)),
                     "state_max_rel": float(np.abs(U - Uo).max() / np.abs(Uo).max()),
                     "linear_iterations_equal": bool(np.array_equal(h[:, 12], ho[:, 12]))}
    return out


def run_warmstart(args, wl, torch, mesh, clocks):
    """Train the warm start on the batched solver's states and compare, on held-out
    conditions, the iterations needed to reach a residual target from the prediction and from
    the freestream.  value: cell-updates/s of the held-out batch started from the prediction."""
    from bes_gb300 import lib, meshgen

    def machs(seed, n):
        return np.array([meshgen.freestream_mach_vector(*c)
                         for c in meshgen.sample_conditions(n, seed)])

    opts = lib.default_options(**wl["opts"])
    train, test = machs(*wl["train"]), machs(*wl["test"])
    t0 = time.perf_counter()
    data = lib.Context(mesh, opts, machs=train)
    data.explicit_iterations(wl["data_iters"], history=False)
    states = data.get_state()
    data.close()
    t_data = time.perf_counter() - t0
    base = lib.Context(mesh, opts)
    net = lib.WarmStart(base, seed=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = net.train(train, states, steps=wl["train_steps"], batch=wl["batch"], lr=1e-3,
                     weight_decay=1e-4, seed=1)
    t_train = time.perf_counter() - t0
    n_it = wl["eval_iters"]
    fs = lib.Context(mesh, opts, machs=test)
    h_fs = fs.explicit_iterations(n_it)
    U_ref = fs.get_state()
    fs.close()
    warm = lib.Context(mesh, opts, machs=test)
    used = net.init_state(warm)
    U0 = warm.get_state()
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h_w = warm.explicit_iterations(n_it)
    torch.cuda.synchronize()
    t_warm = time.perf_counter() - t0
    clk = clocks.stop()
    r_fs = np.sqrt((h_fs[:, :, :5] ** 2).sum(axis=2))
    r_w = np.sqrt((h_w[:, :, :5] ** 2).sum(axis=2))
    target = r_fs[n_it // 2]
    it_fs = [int(np.argmax(r_fs[:, b] <= target[b]) + 1) for b in range(len(test))]
    it_w = [int(np.argmax(r_w[:, b] <= target[b]) + 1) if (r_w[:, b] <= target[b]).any()
            else None for b in range(len(test))]
    err_pred = np.linalg.norm((U0 - U_ref).reshape(len(test), -1), axis=1) / \
        np.linalg.norm(U_ref.reshape(len(test), -1), axis=1)
    nc = warm.n_cells
    warm.close()
    net.close()
    base.close()
    value = len(test) * nc * n_it / t_warm
    return {"metric": METRIC, "metric_full": METRIC_FULL, "value": value, "unit": METRIC,
            "n_gpus": 1, "steps": n_it, "warmup": 0, "ms_per_step": t_warm / n_it * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": args.workload, "cells": nc, "train_conditions": len(train),
                       "test_conditions": len(test), "parallelism": "replicas1",
                       "l2": "not flushed (wall clock of a whole batched run)"},
            "warm_start": {
                "iterations_to_target_freestream": it_fs, "iterations_to_target_warm": it_w,
                "target": "the freestream run's residual L2 at iteration %d" % (n_it // 2),
                "prediction_rel_error_vs_state_at_%d" % n_it: [float(x) for x in err_pred],
                "prediction_used": [int(x) for x in used],
                "train_seconds": t_train, "data_seconds": t_data,
                "final_loss": float(loss[-100:].mean()), "first_loss": float(loss[:10].mean())},
            "clocks": clk}


def _solve_to(ctx, target, max_steps):
    """Implicit steps until the unscaled residual L2 (all variables) is <= target; returns
    (steps, seconds, first residual, last residual)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r0 = r = None
    steps = 0
    for _ in range(max_steps):
        h = ctx.implicit_steps(1)[0]
        steps += 1
        r = float(np.sqrt(np.sum(h[14:19] ** 2)))
        if r0 is None:
            r0 = r
        if target is None:
            target = 1e-8 * r0
        if r <= target or not np.isfinite(r):
            break
    torch.cuda.synchronize()
    return steps, time.perf_counter() - t0, r0, r, target


def _freestream_states(machs, nc, gamma=1.4, R=287.0):
    """Step-0 freestream conserved state of each Mach vector, [n, nc, 5]."""
    out = np.zeros((len(machs), nc, 5))
    for q, m in enumerate(machs):
        T = 1.0 / (gamma * R)
        cv = R / (gamma - 1.0)
        u = np.asarray(m, dtype=np.float64)
        out[q, :, 0] = 1.0
        out[q, :, 1:4] = u
        out[q, :, 4] = cv * T + 0.5 * float(u @ u)
    return out


def _physical(U, gamma=1.4):
    p = (gamma - 1.0) * (U[..., 4] - 0.5 * (U[..., 1] ** 2 + U[..., 2] ** 2 + U[..., 3] ** 2)
                         / U[..., 0])
    return bool(np.all(U[..., 0] > 0) and np.all(p > 0) and np.all(np.isfinite(U)))


def run_production(args, wl, torch, mesh, clocks):
    """Learned warm start on the Gaussian-bump box: training data from the batched implicit sweep,
    AdamW training of the FiLM MLP on the GPU, held-out conditions solved from the prediction
    and from the freestream (batched), the plain FP64 solver on a sample; value: cell-updates/s
    of the warm-started sweep."""
    from bes_gb300 import lib, meshgen

    def machs(seed, n):
        return np.array([meshgen.freestream_mach_vector(*c)
                         for c in meshgen.sample_conditions(n, seed)])

    op = dict(wl["opts"], linear_solver_tol=wl["prod_tol"])
    o64 = dict(wl["opts"], precision=0)
    train, test = machs(*wl["train"]), machs(*wl["test"])
    slots = min(wl["slots"], len(train))
    clocks.start()
    # 1. training data: the batched sweep from the freestream to a 1e-8 drop, in chunks of
    # two slot-fills; no new chunk starts after data_budget_s seconds (progress on stderr)
    t0 = time.perf_counter()
    cd = lib.Context(mesh, lib.default_options(**op), machs=train[:slots])
    nc = cd.n_cells
    chunk = 2 * slots
    states, ok_machs, attempted, data_steps = [], [], 0, 0
    for c0 in range(0, len(train), chunk):
        part = train[c0:c0 + chunk]
        d = cd.implicit_sweep(part, drop=1e-8, max_steps=wl["data_max_steps"], states=True)
        conv = d["final_res"] <= 1e-8
        states.extend(d["U"][conv])
        ok_machs.extend(part[conv])
        attempted += len(part)
        data_steps += int(d["steps"].sum())
        del d
        el = time.perf_counter() - t0
        print(json.dumps({"progress": "training data", "attempted": attempted,
                          "converged": len(ok_machs), "seconds": el}), file=sys.stderr,
              flush=True)
        if el > wl.get("data_budget_s", 1e30):
            break
    cd.close()
    t_data = time.perf_counter() - t0
    states = np.array(states)
    ok_machs = np.array(ok_machs)
    # 2. training on the GPU (tcgen05 GEMMs, AdamW)
    base = lib.Context(mesh, lib.default_options(**op))
    net = lib.WarmStart(base, seed=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = net.train(ok_machs, states, steps=wl["train_steps"], batch=wl["batch"], lr=1e-3,
                     weight_decay=1e-4, seed=1)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del states
    # 3. held-out conditions: the freestream state's residual sets each condition's target
    n = len(test)
    ns = min(wl["slots"], n)
    c1 = lib.Context(mesh, lib.default_options(**op), machs=test)
    h1 = c1.implicit_steps(1)
    c1.close()
    r0 = np.sqrt((h1[0, :, 14:19] ** 2).sum(axis=1))
    target = 1e-8 * r0
    pred = net.infer(test)
    used = np.array([_physical(pred[q]) for q in range(n)])
    U0 = np.where(used[:, None, None], pred, _freestream_states(test, nc))
    del pred
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cc = lib.Context(mesh, lib.default_options(**op), machs=test[:ns])
    cold = cc.implicit_sweep(test, target=target, max_steps=wl["max_steps"], states=True)
    cc.close()
    t_cold = time.perf_counter() - t0
    print(json.dumps({"progress": "cold", "converged": int((cold["steps"] < wl["max_steps"]).sum()),
                      "seconds": t_cold}), file=sys.stderr, flush=True)
    # from a predicted field the CFL ramp starts at 100 (10 steps to 1000)
    ow = dict(op, cfl_ramp_start=100.0, cfl_ramp_steps=10)
    t0 = time.perf_counter()
    cw = lib.Context(mesh, lib.default_options(**ow), machs=test[:ns])
    warm = cw.implicit_sweep(test, U0=U0, target=target, max_steps=wl["max_steps"], states=True)
    cw.close()
    t_warm = time.perf_counter() - t0
    print(json.dumps({"progress": "warm", "converged": int((warm["steps"] < wl["max_steps"]).sum()),
                      "seconds": t_warm, "steps_mean": float(warm["steps"].mean()),
                      "cold_steps_mean": float(cold["steps"].mean())}), file=sys.stderr,
          flush=True)
    # the plain FP64 solver, one condition per context, on a sample
    npl = min(n, wl["plain_sample"])
    t0 = time.perf_counter()
    c64 = lib.Context(mesh, lib.default_options(**dict(o64, freestream_mach=tuple(test[0]))))
    plain = c64.implicit_sweep(test[:npl], target=target[:npl], max_steps=wl["max_steps"],
                               states=True)
    c64.close()
    t_plain = time.perf_counter() - t0
    clk = clocks.stop()
    # a solve that stopped before the step limit with a finite residual met its target (the
    # final residuals are relative to each run's own first residual, which for a run from the
    # prediction is not the freestream's)
    lim = wl["max_steps"]
    met = lambda out: (out["steps"] < lim) & np.isfinite(out["final_res"])
    conv_c, conv_w, conv_p = met(cold), met(warm), met(plain)
    qd = 0.5 * (test ** 2).sum(axis=1)
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    rows = []
    for q in range(n):
        r = dict(mach=[float(x) for x in test[q]], prediction_used=bool(used[q]),
                 cold_steps=int(cold["steps"][q]), warm_steps=int(warm["steps"][q]),
                 cold_converged=bool(conv_c[q]), warm_converged=bool(conv_w[q]),
                 prediction_rel_l2_vs_cold=rel(U0[q], cold["U"][q]),
                 warm_state_rel_l2_vs_cold=rel(warm["U"][q], cold["U"][q]),
                 warm_force_coefficient_abs_diff_vs_cold=float(
                     np.abs(warm["force"][q] - cold["force"][q]).max() / qd[q]))
        if q < npl:
            r.update(plain_steps=int(plain["steps"][q]), plain_converged=bool(conv_p[q]),
                     cold_state_rel_l2_vs_fp64=rel(cold["U"][q], plain["U"][q]),
                     warm_state_rel_l2_vs_fp64=rel(warm["U"][q], plain["U"][q]),
                     cold_force_coefficient_abs_diff_vs_fp64=float(
                         np.abs(cold["force"][q] - plain["force"][q]).max() / qd[q]),
                     warm_force_coefficient_abs_diff_vs_fp64=float(
                         np.abs(warm["force"][q] - plain["force"][q]).max() / qd[q]))
        rows.append(r)
    both = [r for r in rows if r["cold_converged"] and r["warm_converged"]]
    same = [r for r in both if r["warm_state_rel_l2_vs_cold"] < 1e-6]
    sph = lambda k, t: 3600.0 * int(k.sum()) / t
    net.close()
    base.close()
    steps_w = int(warm["steps"].sum())
    return {"metric": METRIC, "metric_full": METRIC_FULL,
            "value": nc * steps_w / t_warm, "unit": METRIC, "n_gpus": 1,
            "steps": steps_w, "warmup": 0, "ms_per_step": t_warm / steps_w * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 system stored as fp16 blocks, fp16 Krylov basis / f64 residual and "
                     "update; network bf16 GEMMs (tcgen05) with fp32 accumulation",
            "data": "synthetic",
            "config": {"workload": args.workload, "cells": nc, "slots": ns,
                       "train_conditions": len(train), "train_attempted": attempted,
                       "train_converged": len(ok_machs), "train_data_steps": data_steps,
                       "test_conditions": n, "plain_sample": npl,
                       "train_steps": wl["train_steps"], "batch": wl["batch"],
                       "production_linear_tol": wl["prod_tol"], "parallelism": "replicas1",
                       "l2": "not flushed (wall clock of whole solves)"},
            "warm_start": {
                "steps_to_target": {"warm_mean": float(warm["steps"].mean()),
                                    "cold_mean": float(cold["steps"].mean()),
                                    "warm_mean_converged_both": float(np.mean([r["warm_steps"] for r in both])) if both else None,
                                    "cold_mean_converged_both": float(np.mean([r["cold_steps"] for r in both])) if both else None},
                "seconds": {"warm_batched": t_warm, "cold_batched": t_cold,
                            "plain_fp64_sample": t_plain, "training_data": t_data,
                            "training": t_train},
                "converged": {"warm": int(conv_w.sum()), "cold": int(conv_c.sum()), "of": n,
                              "plain_fp64": int(conv_p.sum()), "plain_of": npl},
                "solves_per_hour": {"warm_batched": sph(conv_w, t_warm),
                                    "cold_batched": sph(conv_c, t_cold),
                                    "plain_fp64": sph(conv_p, t_plain)},
                "same_steady_state_as_cold": {"count": len(same), "of_converged_both": len(both)},
                "prediction_used": int(used.sum()),
                "loss_first_last": [float(loss[:10].mean()), float(loss[-100:].mean())],
                "target": "1e-8 x the freestream state's residual L2, per condition"},
            "per_condition": rows, "clocks": clk}


def run_isweep(args, wl, torch, mesh, clocks):
    """Converged solves/hour of a batched implicit sweep against the plain FP64 solver.
    value: cell-updates/s of the batched production sweep (cells x steps of every condition /
    wall time of the whole sweep); converged_sweep: solves/hour of both forms, their ratio and
    the force-coefficient differences on the conditions both solved.  The production form runs
    every condition; the plain FP64 solver runs a sample of the conditions the production form
    converged (the first `plain_sample` of them; the first conditions if it converged none), so
    the plain solver is not charged for the conditions the scheme does not converge."""
    from bes_gb300 import lib, meshgen
    seed, n = wl["conds"]
    machs = np.array([meshgen.freestream_mach_vector(*c)
                      for c in meshgen.sample_conditions(n, seed)])
    nplain = min(n, wl["plain_sample"])
    o64 = dict(wl["opts"], precision=0)
    op = dict(wl["opts"], linear_solver_tol=wl["prod_tol"])
    nc = int(mesh.n_cells)
    clocks.start()
    # production: every condition through the slots of one batched context
    slots = min(n, wl["slots"])
    free, _ = torch.cuda.mem_get_info()
    per_slot, shared = 1300.0 * nc, 3000.0 * nc  # bytes, with margin (implicit_allocate)
    slots = max(1, min(slots, int((free - 8e9 - shared) // per_slot)))
    cb = lib.Context(mesh, lib.default_options(**op), machs=machs[:slots])
    used = free - torch.cuda.mem_get_info()[0]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s0 = cb.implicit_stats()
    b = cb.implicit_sweep(machs, drop=1e-8, max_steps=wl["max_steps"])
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    s1 = cb.implicit_stats()
    tuning = cb.tuning().strip()
    cb.close()
    conv_b = b["final_res"] <= 1e-8
    # plain: the FP64 system, one condition per context, from the freestream
    pick = np.flatnonzero(conv_b)[:nplain]
    if len(pick) == 0:
        pick = np.arange(nplain)
    c64 = lib.Context(mesh, lib.default_options(**dict(o64, freestream_mach=tuple(machs[pick[0]]))))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    p = c64.implicit_sweep(machs[pick], drop=1e-8, max_steps=wl["max_steps"])
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    c64.close()
    clk = clocks.stop()
    conv_p = p["final_res"] <= 1e-8
    sph_p = 3600.0 * conv_p.sum() / t_plain
    sph_b = 3600.0 * conv_b.sum() / t_batch
    rows = []
    for k, q in enumerate(pick):
        qd = 0.5 * float(np.sum(machs[q] ** 2))  # dynamic pressure (rho = 1, A_ref = 1)
        rows.append(dict(condition=int(q), mach=[float(x) for x in machs[q]],
                         plain_steps=int(p["steps"][k]), plain_seconds=float(p["seconds"][k]),
                         plain_converged=bool(conv_p[k]),
                         plain_final_drop=float(p["final_res"][k]),
                         batched_final_drop=float(b["final_res"][q]),
                         batched_steps=int(b["steps"][q]),
                         batched_converged=bool(conv_b[q]),
                         force_coefficient_abs_diff=float(np.abs(b["force"][q] - p["force"][k]).max() / qd)))
    both = [r for r in rows if r["plain_converged"] and r["batched_converged"]]
    steps_b = int(b["steps"].sum())
    return {"metric": METRIC, "metric_full": METRIC_FULL,
            "value": nc * steps_b / t_batch, "unit": METRIC, "n_gpus": 1,
            "steps": steps_b, "warmup": 0, "ms_per_step": t_batch / steps_b * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 system stored as fp16 blocks, fp16 Krylov basis / f64 residual and "
                     "update", "data": "synthetic",
            "config": {"workload": args.workload, "cells": nc, "conditions": n, "slots": slots,
                       "device_bytes": int(used), "parallelism": "replicas1",
                       "production_linear_tol": wl["prod_tol"],
                       "l2": "not flushed (wall clock of whole solves)"},
            "converged_sweep": {
                "solves_per_hour": {"batched_fp32_system": sph_b, "plain_fp64": sph_p,
                                    "ratio": sph_b / sph_p if sph_p else None},
                "converged": {"batched_fp32_system": int(conv_b.sum()), "of": n,
                              "plain_fp64": int(conv_p.sum()), "plain_of": len(pick),
                              "plain_sample": "conditions the batched form converged"
                              if conv_b.any() else "the first conditions"},
                "seconds": {"batched_fp32_system": t_batch, "plain_fp64": t_plain},
                "batched_steps_per_condition": [int(x) for x in b["steps"]],
                "batched_final_drop_per_condition": [float(x) for x in b["final_res"]],
                "host_syncs": s1["host_syncs"] - s0["host_syncs"],
                "tuning": tuning,
                "max_force_coefficient_abs_diff": (max(r["force_coefficient_abs_diff"] for r in both)
                                                   if both else None),
                "target": "1e-8 x each condition's first residual L2 (both start from the "
                          "freestream)"},
            "per_condition_sampled": rows, "clocks": clk}


# Device bytes per cell of a batched implicit context with the 16-bit storage (precision 2):
# per slot (state, face-side states, fluxes, time steps, the 16-bit matrix, factors and
# inverse diagonal, the FP16 basis of 31 vectors, the FP32 and FP64 Krylov vectors: about
# 1.26 kB, rounded up) and shared by the slots (mesh and geometry, the FP32 assembly and
# factorisation scratch: about 1.9 kB, rounded up)
SLOT_BYTES_PER_CELL = 1350
SHARED_BYTES_PER_CELL = 2200


def run_scale(args, wl, torch, mesh, clocks):
    """Batched implicit steps of many conditions on a large mesh: one step = one graph launch
    advancing every slot of the context; value = slots x cells x steps / event-timed device
    time.  The slots are the first of the workload's conditions, as many as the device memory
    holds.  Reports the device memory the context holds and its set-up time (host mesh build,
    renumbering, upload)."""
    from bes_gb300 import lib, meshgen
    seed, n_drawn = wl["conds"]
    free0, total = torch.cuda.mem_get_info()
    nc_mesh = int(mesh.n_cells)
    fit = int((free0 - 8e9 - SHARED_BYTES_PER_CELL * nc_mesh) // (SLOT_BYTES_PER_CELL * nc_mesh))
    n = max(1, min(n_drawn, fit))
    machs = np.array([meshgen.freestream_mach_vector(*c)
                      for c in meshgen.sample_conditions(n_drawn, seed)])[:n]
    t0 = time.perf_counter()
    ctx = lib.Context(mesh, lib.default_options(**wl["opts"]), machs=machs)
    t_setup = time.perf_counter() - t0
    ctx.implicit_steps(args.warmup)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    ext = torch.cuda.ExternalStream(ctx.stream_handle)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    c0 = ctx.counters()
    hist = []
    clocks.start()
    for k in range(args.steps):
        starts[k].record(ext)
        hist.append(ctx.implicit_steps(1)[0])
        ends[k].record(ext)
    torch.cuda.synchronize()
    clk = clocks.stop()
    c1 = ctx.counters()
    dev_ms = float(sum(a.elapsed_time(b) for a, b in zip(starts, ends)))
    hist = np.array(hist)  # [steps, n, 19]
    nc = ctx.n_cells
    ctx.close()
    value = n * nc * args.steps / (dev_ms / 1e3)
    return {"metric": METRIC, "metric_full": METRIC_FULL, "value": value, "unit": METRIC,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 system stored as fp16 blocks, fp16 Krylov basis / f64 residual and "
                     "update", "data": "synthetic",
            "config": {"workload": args.workload, "cells": nc, "conditions": n,
                       "conditions_drawn": n_drawn, "parallelism": "replicas1",
                       "l2": "inputs larger than L2 (a step streams tens of GB)",
                       "linear_iterations_per_condition_step": float(hist[:, :, 12].mean()),
                       "device_memory_gb": (free0 - free1) / 1e9,
                       "device_memory_total_gb": total / 1e9,
                       "setup_seconds": t_setup},
            "e2e": None, "gpu_launches": c1["launches"] - c0["launches"], "clocks": clk}


def run_converge(args, wl, ctx, max_steps: int, drop: float = 1e-8):
    """Implicit steps until the L2 of the unscaled residual (all variables) falls by `drop`
    relative to the first step; returns steps, device-synchronous wall time and the history."""
    import torch
    hist = []
    t0 = time.perf_counter()
    r0 = None
    steps = 0
    for _ in range(max_steps):
        h = ctx.implicit_steps(1)[0]
        hist.append(h)
        steps += 1
        r = float(np.sqrt(np.sum(h[14:19] ** 2)))
        if r0 is None:
            r0 = r
        if r <= drop * r0 or not np.isfinite(r):
            break
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    hist = np.array(hist)
    rel = float(np.sqrt(np.sum(hist[-1, 14:19] ** 2)) / r0)
    return dict(steps=steps, seconds=dt, final_drop=rel, converged=bool(rel <= drop),
                linear_iterations=int(hist[:, 12].sum()),
                solves_per_hour=3600.0 / dt if rel <= drop else 0.0,
                wall_force=[float(x) for x in ctx.wall_force()])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--workload", default="implicit_bump_2m", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--converge", type=int, default=-1,
                    help="implicit workloads: also solve to a 1e-8 residual drop from the "
                         "freestream with the FP32 and the FP64 system (max steps; default: "
                         "300 for implicit_bump_2m, 0 = off)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local_rank)

    from bes_gb300 import build as nbuild
    from bes_gb300 import lib
    nbuild.build()
    mesh = make_mesh(wl["mesh"])
    if wl["kind"] in ("warmstart", "production", "scale", "isweep"):
        fn = {"warmstart": run_warmstart, "production": run_production,
              "scale": run_scale, "isweep": run_isweep}[wl["kind"]]
        line = fn(args, wl, torch, mesh, ClockSampler(local_rank))
        if rank == 0:
            print(json.dumps(line))
        return 0
    machs = None
    if "conds" in wl:
        from bes_gb300 import meshgen
        seed, n = wl["conds"]
        machs = np.array([meshgen.freestream_mach_vector(*c)
                          for c in meshgen.sample_conditions(n, seed)])
    ctx = lib.Context(mesh, lib.default_options(**wl["opts"]), machs=machs)
    nc, nf = ctx.n_cells, ctx.n_faces
    ncond = ctx.n_cond
    if wl["kind"] == "implicit":
        line = run_implicit(args, wl, torch, ctx, mesh, world, rank, local_rank, dist)
        n_conv = args.converge if args.converge >= 0 else wl.get("converge", 0)
        if n_conv > 0:
            ctx.close()
            # converged solves/hour to a 1e-8 drop: the FP32-system defect correction against
            # the plain FP64 system, each from the freestream, and their answers compared
            runs = {}
            for name, prec in (("mixed", int(wl["opts"].get("precision", 1)) or 1), ("fp64", 0)):
                o = dict(wl["opts"])
                o["precision"] = prec
                c2 = lib.Context(mesh, lib.default_options(**o))
                runs[name] = run_converge(args, wl, c2, n_conv)
                runs[name]["state"] = c2.get_state()
                c2.close()
            U32, U64 = runs["mixed"].pop("state"), runs["fp64"].pop("state")
            F32 = np.array(runs["mixed"]["wall_force"])
            F64 = np.array(runs["fp64"]["wall_force"])
            line["converged_solve"] = {
                "mixed": runs["mixed"], "fp64": runs["fp64"],
                "solves_per_hour_ratio": (runs["mixed"]["solves_per_hour"]
                                          / runs["fp64"]["solves_per_hour"]
                                          if runs["fp64"]["solves_per_hour"] else None),
                "state_rel_l2_vs_fp64": float(np.linalg.norm(U32 - U64) / np.linalg.norm(U64)),
                "force_abs_diff_vs_fp64": float(np.abs(F32 - F64).max()),
                "force_coefficient_abs_diff_vs_fp64": float(
                    np.abs(F32 - F64).max() / (0.5 * np.sum(np.square(wl["opts"]["freestream_mach"]))))}
            ctx = None
        if ctx is not None:
            ctx.close()
        if rank == 0:
            print(json.dumps(line))
        if dist:
            dist.destroy_process_group()
        return 0

    ctx.enqueue(args.warmup)
    ctx.synchronize()
    ext = torch.cuda.ExternalStream(ctx.stream_handle)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kms = np.zeros(4)
    clocks = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    for k in range(args.steps):
        with torch.cuda.stream(ext):
            flush.fill_(float(k))
            starts[k].record(ext)
        ctx.enqueue(1)
        ends[k].record(ext)
        ext.synchronize()
        t = ctx.last_kernel_times()
        kms += np.array([t["cell_ms"], t["face_ms"], t["update_ms"], t["total_ms"]])
    ctx.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        dist.barrier()
    dev_ms = float(sum(s.elapsed_time(e) for s, e in zip(starts, ends)))
    t_max = max_over_ranks(dev_ms, dist)
    value = world * ncond * nc * args.steps / (t_max / 1e3)

    # end to end through the C ABI with host buffers
    U = ctx.get_state()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.set_state(U)
        ctx.explicit_iterations(1)
        U = ctx.get_state()
    e2e_s = time.perf_counter() - t0
    e2e_max = max_over_ranks(e2e_s, dist)
    e2e = world * ncond * nc * args.steps / e2e_max

    n_stage = 4
    per_launch = {"cell_recon_kernel": kms[0] / (args.steps * n_stage),
                  "face_flux_kernel": kms[1] / (args.steps * n_stage),
                  "update_kernel": kms[2] / (args.steps * n_stage)}
    bytes_per_launch = {"cell_recon_kernel": BYTES_PER_CELL_SWEEP * nc * ncond,
                        "face_flux_kernel": BYTES_PER_FACE * nf * ncond,
                        "update_kernel": BYTES_PER_UPDATE * nc * ncond}
    dom = max(per_launch, key=lambda k: per_launch[k])
    peak, peak_kind = measured_peaks()
    achieved = bytes_per_launch[dom] / (per_launch[dom] / 1e3) / 1e9
    # the explicit kernels move about one FP64 flop per byte, far above this GPU's FP64 ridge
    # point: their bound is the FP64 pipe (counted flops over the measured FMA rate x 2)
    flops_per_launch = {"cell_recon_kernel": (FLOPS_PER_CELL_STAGE - FLOPS_PER_UPDATE
                                              + FLOPS_PER_CELL_DT / n_stage) * nc * ncond,
                        "face_flux_kernel": FLOPS_PER_FACE_STAGE * nf * ncond,
                        "update_kernel": FLOPS_PER_UPDATE * nc * ncond}
    fp64_peak = 2.0 * lib.fp64_fma_rate() / 1e12
    fp64_achieved = flops_per_launch[dom] / (per_launch[dom] / 1e3) / 1e12
    roof = {"kernel": dom, "bound": "fp64", "achieved": fp64_achieved, "peak": fp64_peak,
            "unit": "TFLOP/s", "frac": fp64_achieved / fp64_peak,
            "peak_source": "measured (bes_fp64_fma_rate: independent FP64 FMA chains on every "
                           "SM, 2 flops per FMA)",
            "traffic": traffic_from_profiles(dom, args.workload),
            "ms_per_launch": per_launch[dom], "flops_per_launch": flops_per_launch[dom],
            "hbm": {"achieved_gbs": achieved, "peak_gbs": peak, "frac": achieved / peak,
                    "bytes_per_launch": bytes_per_launch[dom], "peak_source": peak_kind},
            "kernel_ms_per_step": {"cell_recon_kernel": kms[0] / args.steps,
                                   "face_flux_kernel": kms[1] / args.steps,
                                   "update_kernel": kms[2] / args.steps}}
    line = {"metric": METRIC, "metric_full": METRIC_FULL, "value": value, "unit": METRIC,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "cells": nc, "faces": nf,
                       "conditions": ncond, "parallelism": f"replicas{world}",
                       "l2": "flushed before every timed step (256 MB write)"},
            "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": 40 * nc * ncond,
                    "d2h_bytes_per_step": (40 * nc + 80) * ncond + 4},
            "gpu_launches": 14 * args.steps, "roofline": roof,
            "fp64_work": explicit_fp64_work(nc, nf, value / world), "clocks": clk}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl, mesh, mach=None if machs is None else machs[0])
    ctx.close()
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
