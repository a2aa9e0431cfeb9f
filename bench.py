"""Benchmark of the per-step PIC/FLIP + MAC-grid + pressure-projection path.

Workload: the 1024x1024 dam break with a circular solid obstacle (radius 100
cells), ~1.7M marker particles (4 per fluid cell), FLIP ratio 0.95, rho = dt =
0.005, Jacobi-PCG to relative residual 1e-5 -- FluidSolver::stepPICFLIP
(src/FluidSolver.cpp:211-251) per step.  Metric: cell-steps/s (cells x steps /
device time).  A "step" is one stepPICFLIP of the evolving simulation.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

--impl gpu (default) prints one JSON line with the device-time throughput
(`value`), the end-to-end throughput through the C ABI with host particle
buffers (`e2e`: the same steps replayed from the timed region's start state,
the particles uploaded from and downloaded to pinned host memory every step,
wall-clock time), the CG kernel's roofline, the CPU baseline of the same
workload and the SM clocks seen during the timed region.  --impl reference
times the reference's CPU implementation of the path (the reference's own
sources when built here, else the C restatement of them) on the same
workload.  Under torchrun (N > 1) every rank runs an independent replica
(nothing on the data path is exchanged); rank 0 prints.

At N = 1 the line also carries `forms`: the batched form (512 independent
simulations of sides 32..256 stepped as one graph-replayed batch step), the
multigrid form (the same 1024^2 workload with a multigrid-preconditioned
pressure solve, not the reference's solver) and the mixed-precision form (the
4096^2 pressure projection to relative residual 1e-10 by FP64 iterative
refinement around float multigrid or Jacobi CG corrections, against an
FP64-only CG), and the large step (the plain step on the dam break at twice
the side, whose pressure system the CG keeps on chip in its 12-chunk form),
the 500-step trajectory of the workload from its initial state with
per-phase times (the configuration as it is stated), and the per-phase
roofline rows of the dam break at 4096^2.  The batched form also steps the
same members as plain handles one after another (`vs_handles`), and the
mixed-precision form states every method's error against FP64 on the host:
the residual recomputed from the returned solution at 4096^2, and the
distance to an FP64 direct solve at 512^2.  --no-forms skips them;
--only-form measures one of them alone.

Both arms time steps W+1..W+K of the workload (the GPU arm's last warm-up
step records the timed CUDA graph) and carry the same `config`; what
differs between them is under `measurement`.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-steps/s at 1024^2 (CG tol 1e-5)"
UNIT = "cell-steps/s"
CG_BYTES_PER_CELL_ITER = 42  # fused Jacobi-PCG: 17 B (SpMV pass) + 25 B (update pass) per fluid cell
L2_FLUSH_BYTES = 256 << 20


def phase_bytes(n_cells, n_particles, n_fluid, cg_iterations):
    """Algorithmic bytes of each timed phase of one stepPICFLIP: every array
    the phase must read or write, counted once (float grids and particle
    fields 4 B, labels and masks 1 B).  N cells, P particles, F fluid cells,
    I CG iterations; the phases are those of src/FluidSolver.cpp:211-251."""
    N, P, F, I = n_cells, n_particles, n_fluid, cg_iterations
    return {"classify": 8 * P + 2 * N,            # positions in; solid mask in, labels out
            "p2g": 16 * P + 16 * N,               # particles in; u, v and their previous copies out
            "forces": 17 * N,                     # labels in; u, v in and out (gravity, walls, extension)
            "assembly": 8 * P + 13 * N + 13 * F,  # positions in (counts); labels, u, v in; fluid index out;
                                                  # right-hand side, down/up rows, flags out
            "cg": CG_BYTES_PER_CELL_ITER * F * I,
            "project": 37 * N,                    # pressure, labels, u, v in; u, v out; walls; diff out
            "g2p": 32 * P}                        # particles in and out (grid samples hit in cache)


PHASE_MODEL = ("algorithmic bytes per step: classify 8P+2N, p2g 16P+16N, forces 17N, assembly 8P+13N+13F, "
               "cg 42FI, project 37N, g2p 32P")


def per_phase_rows(bytes_sum, ms_sum, steps, peak):
    """{phase: algorithmic bytes and ms per step, GB/s, fraction of peak}."""
    rows = {}
    for k, b in bytes_sum.items():
        ms = ms_sum.get(k, 0.0)
        gbs = b / (ms / 1000.0) / 1e9 if ms > 0 else None
        rows[k] = {"bytes_per_step": int(b / steps), "ms_per_step": ms / steps, "gbs": gbs,
                   "frac": gbs / peak if gbs else None}
    return rows


def fp64_residual(labels, rhs, x):
    """||b - A x|| / ||b|| over the fluid cells in float64, A the reference's
    pressure matrix on unit cells (src/FluidSolver.cpp:363-416: +1 per liquid
    neighbour, minus the count of non-solid neighbours on the diagonal),
    evaluated matrix-free from the label grid."""
    L = np.pad(labels, 1, constant_values=2)
    X = np.pad(np.asarray(x, np.float64), 1)
    fl = labels == 0
    ax = np.zeros(labels.shape)
    cnt = np.zeros(labels.shape)
    ny, nx = labels.shape
    for dj, di in ((0, -1), (0, 1), (-1, 0), (1, 0)):
        nl = L[1 + dj:1 + dj + ny, 1 + di:1 + di + nx]
        xn = X[1 + dj:1 + dj + ny, 1 + di:1 + di + nx]
        ax += np.where(nl == 0, xn, 0.0)
        cnt += nl != 2
    ax -= cnt * x
    b = np.asarray(rhs, np.float64)[fl]
    return float(np.linalg.norm(b - ax[fl]) / np.linalg.norm(b))


def fp64_direct_solution(labels, rhs):
    """FP64 direct solve (scipy spsolve) of the same system: one unknown of
    each connected fluid component pinned, then every component shifted to
    zero mean, where the solution is unique."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    from scipy import ndimage

    fl = labels == 0
    idx = -np.ones(labels.shape, np.int64)
    idx[fl] = np.arange(int(fl.sum()))
    jj, ii = np.nonzero(fl)
    k = idx[jj, ii]
    rows, cols = [k], [k]
    diag = np.zeros(k.size)
    vals = []
    L = np.pad(labels, 1, constant_values=2)
    I = np.pad(idx, 1, constant_values=-1)
    for dj, di in ((0, -1), (0, 1), (-1, 0), (1, 0)):
        nl = L[jj + 1 + dj, ii + 1 + di]
        diag -= nl != 2
        liq = nl == 0
        rows.append(k[liq])
        cols.append(I[jj[liq] + 1 + dj, ii[liq] + 1 + di])
        vals.append(np.ones(int(liq.sum())))
    vals.insert(0, diag)
    n = k.size
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    b = np.asarray(rhs, np.float64)[fl]
    comp, nc = ndimage.label(fl, structure=[[0, 1, 0], [1, 1, 1], [0, 1, 0]])
    cidx = comp[fl]
    _, pins = np.unique(cidx, return_index=True)
    keep = np.ones(n, bool)
    keep[pins] = False
    xd = np.zeros(n)
    xd[keep] = spla.spsolve(A[keep][:, keep].tocsc(), b[keep])
    return demean_components(xd, cidx, nc), cidx, nc


def demean_components(v, cidx, nc):
    from scipy import ndimage

    means = ndimage.mean(v, cidx, index=np.arange(1, nc + 1))
    return v - means[cidx - 1]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--cpu-budget", type=float, default=150.0, help="seconds of CPU work for CPU timings")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample (profiling runs)")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched and mixed-precision forms")
    ap.add_argument("--batch", type=int, default=512, help="members of the batched form")
    ap.add_argument("--projection-size", type=int, default=4096, help="grid side of the mixed-precision form")
    ap.add_argument("--projection-methods", default="mixed_multigrid,mixed_f32_dots,mixed_ds_dots,mixed_f64_dots,fp64",
                    help="solves of the mixed-precision form, in order (also fp32: the step's Jacobi CG alone, "
                         "and fp32_ds_dots: the same with double-single dots)")
    ap.add_argument("--projection-max-iterations", type=int, default=200000,
                    help="CG iteration cap of each projection solve (a small cap makes a short profiling case)")
    ap.add_argument("--batch-plan", type=int, choices=[1, 2, 4, 8], default=None,
                    help="batched form: CG chunks per CTA instead of the autotuner's choice")
    ap.add_argument("--batch-trajectory-steps", type=int, default=100,
                    help="steps of the batched form's trajectory from its initial state (0: skip)")
    ap.add_argument("--handles-steps", type=int, default=5,
                    help="batched form: steps of the same members as plain handles, one after another (0: skip)")
    ap.add_argument("--trajectory-steps", type=int, default=500,
                    help="trajectory form: steps of the workload from its initial state (0: skip)")
    ap.add_argument("--phases-size", type=int, default=4096, help="grid side of the per-phase roofline form (0: skip)")
    ap.add_argument("--smoke-size", type=int, default=256, help="grid side of the differentiable smoke form (0: skip)")
    ap.add_argument("--only-form", choices=["batched", "mixed_precision", "multigrid", "large_step", "trajectory",
                                            "phases", "smoke"], default=None,
                    help="measure one form alone (profiling runs) and print its JSON object")
    return ap.parse_args()


def workload(size):
    from fluid_simulation_gb300 import scenes

    return scenes.dam_break_large(size)


def config_of(sc, extra=None):
    c = {"workload": "dam break %dx%d, solid disc r=%g cells, %d particles (4/fluid cell), FLIP 0.95, "
                     "rho=dt=0.005, Jacobi-PCG rel. residual 1e-5, stepPICFLIP"
                     % (sc.size_x, sc.size_y, sc.meta["disc"][2], sc.particles.shape[0]),
         "cells": sc.cells, "particles": int(sc.particles.shape[0]), "dt": sc.dt,
         "cg_tolerance": sc.cg_tolerance, "method": "stepPICFLIP"}
    if extra:
        c.update(extra)
    return c


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- CPU timings
def cpu_oracle_kind():
    from oracle import pyoracle as po

    return "reference" if po.reference_available() else "restatement"


def cpu_sim_from_state(sc, kind, grids, particles):
    from oracle import pyoracle as po

    o = po.OracleSim(kind, sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio)
    o.set_cg(sc.cg_tolerance, sc.cg_max_iterations)
    o.set_use_stock(False)
    if sc.solid is not None:
        o.set_solid_mask(sc.solid)
    for w, g in enumerate(grids):
        o.set_grid(w, g)
    o.set_particles(particles)
    return o


def time_cpu_steps(o, sc, max_steps, budget_s):
    from oracle import pyoracle as po

    times = []
    t_all = time.perf_counter()
    while len(times) < max_steps:
        t0 = time.perf_counter()
        rc = o.step(po.STEP_PICFLIP, sc.dt)
        times.append(time.perf_counter() - t0)
        assert rc == 0
        if time.perf_counter() - t_all > budget_s:
            break
    return times


def run_reference(args, rank):
    """--impl reference: the reference's CPU implementation on the same workload."""
    if rank != 0:
        return
    from oracle import build_oracle

    build_oracle.build_restatement()
    build_oracle.build_reference()
    kind = cpu_oracle_kind()
    sc = workload(args.size)
    from oracle import pyoracle as po

    o = po.OracleSim(kind, sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio)
    o.set_cg(sc.cg_tolerance, sc.cg_max_iterations)
    if sc.solid is not None:
        o.set_solid_mask(sc.solid)
    o.set_particles(sc.particles)
    budget = args.cpu_budget
    t0 = time.perf_counter()
    warm = 0
    for _ in range(args.warmup):
        if time.perf_counter() - t0 > budget / 3:
            break
        o.step(po.STEP_PICFLIP, sc.dt)
        warm += 1
    times = time_cpu_steps(o, sc, args.steps, budget - (time.perf_counter() - t0))
    total = sum(times)
    value = sc.cells * len(times) / total
    sample = ("steps %d..%d of the workload from its initial state (%d warm-up steps run), single thread"
              % (warm + 1, warm + len(times), warm))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": len(times), "warmup": warm, "ms_per_step": 1000 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded SplitMix64 dam break)",
            "config": config_of(sc),
            "measurement": {"implementation": "reference C++ sources + Eigen-subset stand-in"
                            if kind == "reference" else "C restatement of the reference (port)",
                            "timed_steps": "steps %d..%d of the workload" % (warm + 1, warm + len(times))},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "host_cores": os.cpu_count(),
                             "kind": "reference" if kind == "reference" else "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def max_over_ranks(value: float, device: str) -> float:
    """The largest of every rank's value (the job's time is its slowest
    replica's); `device` holds the exchanged tensor ("cuda:k" under NCCL,
    "cpu" under gloo).  One rank: the value itself."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- GPU arm
def read_traffic():
    """DRAM bytes per CG launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "k_cg_dam_break_1024.md")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        if ln.startswith("traffic_bytes_per_launch:"):
            try:
                return float(ln.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def measure_batched(args, local_rank, plain_value, flush):
    """The batched form: args.batch independent simulations (sides U{32..256},
    random blocks and discs, FLIP ratio U[0.9, 1.0], CG 1e-5) advanced by one
    graph-replayed fs_batch_step per step, after the autotuner picked the CG
    cluster plan.  Same timing discipline as the main line."""
    import torch

    import fluid_simulation_gb300 as fsg
    from fluid_simulation_gb300 import scenes

    sc = scenes.batch_scenes(args.batch)
    cells = sum(s.cells for s in sc)
    b = fsg.FluidBatch.from_scenes(sc, device=local_rank)
    b.step(fsg.STEP_PICFLIP, 0.005)
    if args.batch_plan:
        b.set_tuning(args.batch_plan)
        tuned = {"chunks_per_cta": args.batch_plan, "ms_per_step": None}
    else:
        tuned = b.tune(fsg.STEP_PICFLIP, 0.005, steps=2)
    for _ in range(args.warmup):
        b.step(fsg.STEP_PICFLIP, 0.005)
    b.synchronize()
    stream = torch.cuda.ExternalStream(b.stream(), device=local_rank)
    ms, fi, itmax = [], 0, 0
    l0 = b.kernel_launches()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        b.step(fsg.STEP_PICFLIP, 0.005)
        e1.record(stream)
        b.synchronize()
        ms.append(e0.elapsed_time(e1))
    for s in range(len(sc)):
        st = b.stats(s)
        fi += st["n_fluid"] * st["cg_iterations"]
        itmax = max(itmax, st["cg_iterations"])
    t = sum(ms) / 1000.0
    value = cells * args.steps / t
    launches = int(b.kernel_launches() - l0)
    b.close()
    out = {"workload": "%d simulations, sides U{32..256} (seed 0xC3), %d cells, %d particles, "
                       "stepPICFLIP, CG 1e-5" % (len(sc), cells, sum(len(s.particles) for s in sc)),
           "value": value, "unit": UNIT, "ms_per_step": 1000.0 * t / args.steps, "vs_plain": value / plain_value,
           "cg_plan_chunks_per_cta": tuned["chunks_per_cta"], "tuner_ms_per_step": tuned["ms_per_step"],
           "cg_iterations_max_last_step": itmax, "sum_F_I_last_step": fi, "gpu_launches": launches}
    if args.handles_steps > 0:
        nh = min(args.handles_steps, args.steps)
        h = measure_handles(sc, 1 + args.warmup, nh, local_rank, flush)
        batch_ms = float(np.mean(ms[:nh]))
        out["vs_handles"] = {"workload": "the same members, each a plain FluidSim handle stepped one after "
                                         "another (each handle's step is its own CUDA graph)",
                             "steps": nh, "handles_device_ms_per_step": h["device_ms"],
                             "handles_wall_ms_per_step": h["wall_ms"], "batch_ms_per_step_same_steps": batch_ms,
                             "speedup_device": h["device_ms"] / batch_ms, "speedup_wall": h["wall_ms"] / batch_ms}
    if args.batch_trajectory_steps > 0:
        out["trajectory"] = measure_batch_trajectory(sc, cells, args.batch_trajectory_steps, local_rank, flush)
    return out


def measure_batch_trajectory(sc, cells, n, local_rank, flush):
    """The batched configuration as it states it: n (100) steps of a fresh
    batch from the members' initial states, per-step device time.  The cluster
    plan is sized from fluid counts, which exist once a step has classified the
    cells, so step 1 runs on the default plan; the tuner then runs (it leaves
    the state as it found it, and its time is not a step's) and steps 2..n use
    its choice.  Step 1 also captures the step's graph, and so does step 2 for
    the new plan."""
    import torch

    import fluid_simulation_gb300 as fsg

    b = fsg.FluidBatch.from_scenes(sc, device=local_rank)
    stream = torch.cuda.ExternalStream(b.stream(), device=local_rank)
    ms, itmax, tuned = [], {}, None
    for k in range(n):
        if k == 1:
            tuned = b.tune(fsg.STEP_PICFLIP, 0.005, steps=2)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        b.step(fsg.STEP_PICFLIP, 0.005)
        e1.record(stream)
        b.synchronize()
        ms.append(e0.elapsed_time(e1))
        if k in (0, n // 2, n - 1):
            itmax[k + 1] = max(b.stats(m)["cg_iterations"] for m in range(len(sc)))
    b.close()
    t = sum(ms) / 1000.0
    return {"workload": "the batched workload, steps 1..%d from its initial state, tuned after step 1" % n,
            "steps": n, "value": cells * n / t, "unit": UNIT, "ms_per_step": 1000.0 * t / n,
            "ms_step_1": ms[0], "ms_per_step_after_first": float(np.mean(ms[1:])) if n > 1 else None,
            "cg_plan_chunks_per_cta": tuned["chunks_per_cta"] if tuned else None,
            "cg_iterations_max_at_step": itmax}


def measure_handles(scs, pre_steps, steps, local_rank, flush):
    """The batch's members as independent FluidSim handles, stepped one after
    another: pre_steps untimed steps each (the batch's first step and
    warm-up), then `steps` timed steps; per step the sum over members of
    each member's device time (events on its own stream, the member
    synchronised before the next starts) and the wall time of the loop."""
    import torch

    import fluid_simulation_gb300 as fsg

    sims = [fsg.FluidSim.from_scene(sc, device=local_rank) for sc in scs]
    for sim in sims:
        for _ in range(pre_steps):
            sim.step(fsg.STEP_PICFLIP, 0.005)
    torch.cuda.synchronize()
    dev, wall = 0.0, 0.0
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in sims]
    streams = [torch.cuda.ExternalStream(sim.stream(), device=local_rank) for sim in sims]
    for _ in range(steps):
        with torch.cuda.stream(streams[0]):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for sim, (e0, e1), st in zip(sims, evs, streams):
            e0.record(st)
            sim.step(fsg.STEP_PICFLIP, 0.005)
            e1.record(st)
            e1.synchronize()
        wall += time.perf_counter() - t0
        dev += sum(e0.elapsed_time(e1) for e0, e1 in evs)
    for sim in sims:
        sim.close()
    return {"device_ms": dev / steps, "wall_ms": 1000.0 * wall / steps}


def measure_projection(args, local_rank):
    """The mixed-precision form: the pressure projection alone on an n x n
    domain (solid border, 5% random solids, N(0,1) right-hand side with each
    component's mean removed) to relative residual 1e-10, by FP64 iterative
    refinement around float-vector CG (float or double dot products), and by
    an FP64-only CG; device time of each solve."""
    import fluid_simulation_gb300 as fsg
    from fluid_simulation_gb300 import scenes

    n = args.projection_size
    labels, rhs = scenes.projection_problem(n)
    ps = fsg.PoissonSolver(n, n, float(n), float(n), device=local_rank)
    ps.set_problem(labels, rhs)
    out = {"workload": "%dx%d projection, 5%% solids, N(0,1) rhs, relative residual 1e-10" % (n, n),
           "fluid_cells": int((labels == 0).sum())}
    methods = {"mixed_multigrid": (fsg.POISSON_MIXED_MG, fsg.CG_FLOAT),
               "mixed_f32_dots": (fsg.POISSON_MIXED, fsg.CG_FLOAT),
               "mixed_f64_dots": (fsg.POISSON_MIXED, fsg.CG_DOUBLE),
               "mixed_ds_dots": (fsg.POISSON_MIXED, fsg.CG_DS),
               "fp64": (fsg.POISSON_FP64, fsg.CG_FLOAT),
               "fp32": (fsg.POISSON_FP32, fsg.CG_FLOAT),
               "fp32_ds_dots": (fsg.POISSON_FP32, fsg.CG_DS)}
    sols = {}
    for name in args.projection_methods.split(","):
        method, inner = methods[name]
        st = ps.solve(method, 1e-10, args.projection_max_iterations, inner_tol=1e-3, inner_precision=inner)
        x = ps.solution()
        if name in ("mixed_ds_dots", "mixed_f64_dots"):
            sols[name] = x
        out[name] = {"ms": st["ms"], "residual": st["residual"],
                     "residual_fp64_host": fp64_residual(labels, rhs, x),
                     "outer_iterations": st["outer_iterations"], "inner_iterations": st["inner_iterations"],
                     "cell_solves_per_s": n * n / (st["ms"] / 1000.0)}
    out["residual_fp64_host"] = ("||b - A x|| / ||b|| recomputed in float64 on the host from the returned x "
                                 "(numpy, matrix-free), beside the library's own residual")
    if "fp64" in out:
        for name, key in (("mixed_f32_dots", "speedup_mixed_vs_fp64"),
                          ("mixed_multigrid", "speedup_mixed_multigrid_vs_fp64"),
                          ("mixed_f64_dots", "speedup_mixed_f64_dots_vs_fp64")):
            if name in out:
                out[key] = out["fp64"]["ms"] / out[name]["ms"]
        if "mixed_ds_dots" in out:
            out["speedup_mixed_ds_dots_vs_fp64"] = out["fp64"]["ms"] / out["mixed_ds_dots"]["ms"]
    if len(sols) == 2:
        a, b = sols["mixed_ds_dots"], sols["mixed_f64_dots"]
        out["ds_vs_f64_dots_max_rel_diff"] = float(np.abs(a - b).max() / np.abs(b).max())
    ps.close()
    out["fp64_direct_512"] = projection_vs_direct(512, methods, args, local_rank)
    return out


def projection_vs_direct(n, methods, args, local_rank):
    """Every projection method on the n x n problem against an FP64 direct
    solve on the host (both shifted to zero mean per fluid component, where
    the solution is unique): max |x - x_FP64| / max |x_FP64| and the relative
    L2 error."""
    import fluid_simulation_gb300 as fsg
    from fluid_simulation_gb300 import scenes

    labels, rhs = scenes.projection_problem(n)
    t0 = time.perf_counter()
    xd, cidx, nc = fp64_direct_solution(labels, rhs)
    out = {"workload": "%dx%d projection (same generator), relative residual 1e-10 (fp32: 1e-5)" % (n, n),
           "direct_solve_s": time.perf_counter() - t0}
    fl = labels == 0
    ps = fsg.PoissonSolver(n, n, float(n), float(n), device=local_rank)
    ps.set_problem(labels, rhs)
    for name in args.projection_methods.split(","):
        method, inner = methods[name]
        tol = 1e-5 if method == fsg.POISSON_FP32 else 1e-10
        st = ps.solve(method, tol, args.projection_max_iterations, inner_tol=1e-3, inner_precision=inner)
        x = demean_components(ps.solution()[fl], cidx, nc)
        out[name] = {"max_rel_err": float(np.abs(x - xd).max() / np.abs(xd).max()),
                     "l2_rel_err": float(np.linalg.norm(x - xd) / np.linalg.norm(xd)),
                     "residual": st["residual"]}
    ps.close()
    return out


def measure_multigrid(args, local_rank, plain_value, flush):
    """The 1024^2 workload stepped with the multigrid-preconditioned pressure
    solver (FS_SOLVER_MGPCG) to the same relative residual: not the
    reference's pressure, reported beside the bit-exact plain path."""
    import torch

    import fluid_simulation_gb300 as fsg

    sc = workload(args.size)
    sim = fsg.FluidSim.from_scene(sc, device=local_rank)
    sim.set_pressure_solver(fsg.SOLVER_MGPCG)
    for _ in range(args.warmup):
        sim.step(fsg.STEP_PICFLIP, sc.dt)
    sim.synchronize()
    stream = torch.cuda.ExternalStream(sim.stream(), device=local_rank)
    ms, its = [], []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        sim.step(fsg.STEP_PICFLIP, sc.dt)
        e1.record(stream)
        st = sim.stats()
        ms.append(e0.elapsed_time(e1))
        its.append(st["cg_iterations"])
    t = sum(ms) / 1000.0
    value = sc.cells * args.steps / t
    return {"workload": "the plain workload with the multigrid-preconditioned CG (not the reference's solver): the "
                        "mixed-precision step, float vectors and smoothers with double dot products",
            "value": value, "unit": UNIT, "ms_per_step": 1000.0 * t / args.steps, "vs_plain": value / plain_value,
            "cg_iterations_mean": float(np.mean(its))}


def _timed_steps(sim, sc, stream, flush, steps):
    """`steps` stepPICFLIP steps, each timed with CUDA events (an L2-flushing
    write before each, outside the events), with the library's per-phase
    times and the per-phase algorithmic bytes."""
    import torch

    import fluid_simulation_gb300 as fsg

    ms, its = [], []
    phases = {k: 0.0 for k in fsg.TIMED_PHASES}
    bsum = {k: 0 for k in fsg.TIMED_PHASES}
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        sim.step(fsg.STEP_PICFLIP, sc.dt)
        e1.record(stream)
        st = sim.stats()
        ms.append(e0.elapsed_time(e1))
        its.append(st["cg_iterations"])
        for k, v in st["ms_phase"].items():
            phases[k] += v
        for k, v in phase_bytes(sc.cells, sim.num_particles(), st["n_fluid"], st["cg_iterations"]).items():
            bsum[k] += v
    return ms, its, phases, bsum


def measure_trajectory(args, local_rank, flush, peak):
    """The workload as its configuration states it: --trajectory-steps (500)
    stepPICFLIP steps from the initial state on a fresh handle, per-step
    device time, per-phase times and the CG iterations of every step."""
    import torch

    import fluid_simulation_gb300 as fsg

    sc = workload(args.size)
    sim = fsg.FluidSim.from_scene(sc, device=local_rank)
    sim.set_timing(True)
    stream = torch.cuda.ExternalStream(sim.stream(), device=local_rank)
    n = args.trajectory_steps
    t0 = time.perf_counter()
    ms, its, phases, bsum = _timed_steps(sim, sc, stream, flush, n)
    wall = time.perf_counter() - t0
    sim.close()
    t = sum(ms) / 1000.0
    return {"workload": "the plain workload, steps 1..%d from its initial state (the configuration's trajectory)"
                        % n, "steps": n, "value": sc.cells * n / t, "unit": UNIT, "ms_per_step": 1000.0 * t / n,
            "ms_per_step_after_first": float(np.mean(ms[1:])) if n > 1 else None,
            "wall_s": wall, "phases_ms_per_step": {k: v / n for k, v in phases.items()},
            "cg_iterations_mean": float(np.mean(its)), "cg_iterations_max": int(np.max(its)),
            "per_phase_roofline": per_phase_rows(bsum, phases, n, peak), "per_phase_model": PHASE_MODEL}


def measure_smoke(args, local_rank):
    """The differentiable-smoke form: --smoke-size (256)^2, a Gaussian blob in
    seeded Fourier-mode velocity, 64 RK2 steps at dt = 0.01 with the mixed
    projection to 1e-10 (FP64 refinement around Jacobi- or multigrid-
    preconditioned float corrections), checkpoints every 8 steps; the forward
    pass (loss) and the backward pass (gradient of the loss with respect to
    the initial u, v and density, read back to the host), each timed by the
    host clock after one untimed forward + backward."""
    import fluid_simulation_gb300 as fsg
    from fluid_simulation_gb300 import scenes

    n, steps, dt = args.smoke_size, 64, 0.01
    u, v, d, t = scenes.smoke_problem(n)
    out = {"workload": "smoke %dx%d, Gaussian blob (sigma 20), Fourier-mode velocity k<=8, %d RK2 steps at dt=%g, "
                       "projection to 1e-10, checkpoints every 8 steps" % (n, n, steps, dt)}
    for name, prec, proj in (("fp32", fsg.SMOKE_FP32, fsg.POISSON_MIXED),
                             ("fp32_trace64", fsg.SMOKE_FP32_TRACE64, fsg.POISSON_MIXED),
                             ("fp64", fsg.SMOKE_FP64, fsg.POISSON_MIXED),
                             ("fp32_trace64_multigrid", fsg.SMOKE_FP32_TRACE64, fsg.POISSON_MIXED_MG),
                             ("fp64_multigrid", fsg.SMOKE_FP64, fsg.POISSON_MIXED_MG)):
        sm = fsg.Smoke(n, n, dt=dt, integrator=fsg.INTEGRATOR_RK2, precision=prec, projection_method=proj,
                       cg_tolerance=1e-10, checkpoint_every=8, device=local_rank)
        sm.set_state(u, v, d)
        sm.set_target(t)
        sm.forward(steps)
        sm.backward()
        sm.set_state(u, v, d)
        t0 = time.perf_counter()
        loss = sm.forward(steps)
        t1 = time.perf_counter()
        sm.backward()
        t2 = time.perf_counter()
        sm.close()
        out[name] = {"loss": loss, "forward_ms": 1000.0 * (t1 - t0), "backward_ms": 1000.0 * (t2 - t1),
                     "forward_cell_steps_per_s": n * n * steps / (t1 - t0)}
    return out


def measure_phases(args, local_rank, flush, peak):
    """Per-phase roofline rows of the plain step on the dam break at
    --phases-size (4096^2: about 6.9M fluid cells and 27M particles): 2
    warm-up steps, then 2 steps timed with the library's phase events."""
    import torch

    import fluid_simulation_gb300 as fsg

    sc = workload(args.phases_size)
    try:
        sim = fsg.FluidSim.from_scene(sc, device=local_rank)
    except fsg.FsError as e:
        if e.code != 5:  # FS_ERR_TOO_LARGE: the library's own size limit
            raise
        return {"skipped": "the library refused the %dx%d grid: %s" % (sc.size_x, sc.size_y, e)}
    for _ in range(2):
        sim.step(fsg.STEP_PICFLIP, sc.dt)
    sim.set_timing(True)
    stream = torch.cuda.ExternalStream(sim.stream(), device=local_rank)
    ms, its, phases, bsum = _timed_steps(sim, sc, stream, flush, 2)
    nf = sim.stats()["n_fluid"]
    sim.close()
    return {"workload": "dam break %dx%d (the plain workload scaled), %d particles, stepPICFLIP, Jacobi-PCG 1e-5"
                        % (sc.size_x, sc.size_y, sc.particles.shape[0]), "fluid_cells": nf,
            "ms_per_step": float(np.mean(ms)), "cg_iterations": its,
            "per_phase_roofline": per_phase_rows(bsum, phases, 2, peak), "per_phase_model": PHASE_MODEL}


def measure_large_step(args, local_rank, flush):
    """The plain step (the reference's algorithm, bit-exact) on the dam break
    at twice the side, 2048^2: about 1.72M fluid cells, 12 chunks of 1024
    cells per CTA, a system the CG keeps on chip in k_cg_large.  Device time
    per step, and the CG's share from the library's per-phase events."""
    import torch

    import fluid_simulation_gb300 as fsg

    sc = workload(2 * args.size)
    try:
        sim = fsg.FluidSim.from_scene(sc, device=local_rank)
    except fsg.FsError as e:
        if e.code != 5:  # FS_ERR_TOO_LARGE: the library's own size limit
            raise
        return {"skipped": "the library refused the %dx%d grid: %s" % (sc.size_x, sc.size_y, e)}
    for _ in range(2):
        sim.step(fsg.STEP_PICFLIP, sc.dt)
    sim.synchronize()
    sim.set_timing(True)
    stream = torch.cuda.ExternalStream(sim.stream(), device=local_rank)
    ms, cg_ms, its, nf = [], [], [], 0
    for _ in range(3):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        sim.step(fsg.STEP_PICFLIP, sc.dt)
        e1.record(stream)
        st = sim.stats()
        ms.append(e0.elapsed_time(e1))
        cg_ms.append(st["ms_phase"]["cg"])
        its.append(st["cg_iterations"])
        nf = st["n_fluid"]
    sim.set_timing(False)
    t = sum(ms) / 1000.0
    return {"workload": "dam break %dx%d (the plain workload at twice the side), stepPICFLIP, Jacobi-PCG 1e-5"
            % (sc.size_x, sc.size_y), "value": sc.cells * len(ms) / t, "unit": UNIT,
            "ms_per_step": 1000.0 * t / len(ms), "fluid_cells": int(nf), "cg_iterations_mean": float(np.mean(its)),
            "cg_us_per_iteration": 1000.0 * sum(cg_ms) / sum(its)}


def run_gpu(args, rank, world, local_rank):
    import torch

    import fluid_simulation_gb300 as fsg
    from fluid_simulation_gb300 import build as fsbuild

    if rank == 0 or not os.path.exists(fsg.library_path()):
        fsbuild.build()
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    torch.cuda.set_device(local_rank)
    if args.only_form:
        if rank == 0:
            flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda:%d" % local_rank)
            if args.only_form == "batched":
                out = measure_batched(args, local_rank, float("nan"), flush)
            elif args.only_form == "multigrid":
                out = measure_multigrid(args, local_rank, float("nan"), flush)
            elif args.only_form == "large_step":
                out = measure_large_step(args, local_rank, flush)
            elif args.only_form == "trajectory":
                out = measure_trajectory(args, local_rank, flush, peaks()[0])
            elif args.only_form == "phases":
                out = measure_phases(args, local_rank, flush, peaks()[0])
            elif args.only_form == "smoke":
                out = measure_smoke(args, local_rank)
            else:
                out = measure_projection(args, local_rank)
            print(json.dumps({"form": args.only_form, **out}), flush=True)
        return
    sc = workload(args.size)
    sim = fsg.FluidSim.from_scene(sc, device=local_rank)
    stream = torch.cuda.ExternalStream(sim.stream(), device=local_rank)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda:%d" % local_rank)

    # W untimed warm-up steps, the last of which records the timed graph
    # variant (per-phase events): the timed steps are W+1..W+K, as in the
    # reference arm
    for _ in range(max(args.warmup - 1, 0)):
        sim.step(fsg.STEP_PICFLIP, sc.dt)
    sim.set_timing(True)
    if args.warmup > 0:
        sim.step(fsg.STEP_PICFLIP, sc.dt)
    sim.synchronize()
    # state at the start of the timed region, for the CPU baseline sample
    grids0 = [sim.grid(w) for w in range(8)] if rank == 0 else None
    parts0 = sim.particles() if rank == 0 else None
    start = sim.snapshot()  # the end-to-end run below replays the timed steps from here
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    torch.cuda.synchronize()
    step_ms, cg_ms, fi, iters, phases = [], [], 0, [], {k: 0.0 for k in fsg.TIMED_PHASES}
    bsum = {k: 0 for k in fsg.TIMED_PHASES}
    launches0 = sim.kernel_launches()
    with ClockSampler(local_rank) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            sim.step(fsg.STEP_PICFLIP, sc.dt)
            e1.record(stream)
            st = sim.stats()  # synchronises; outside the events
            step_ms.append(e0.elapsed_time(e1))
            cg_ms.append(st["ms_phase"]["cg"])
            for k, v in st["ms_phase"].items():
                phases[k] += v
            fi += st["n_fluid"] * st["cg_iterations"]
            iters.append(st["cg_iterations"])
            for k, v in phase_bytes(sc.cells, sim.num_particles(), st["n_fluid"], st["cg_iterations"]).items():
                bsum[k] += v
    launches = sim.kernel_launches() - launches0
    torch.cuda.synchronize()
    t_dev = max_over_ranks(sum(step_ms) / 1000.0, "cuda:%d" % local_rank)
    value = sc.cells * args.steps * world / t_dev

    # end to end through the C ABI with host (pinned) particle buffers: the same
    # steps as the timed region (replayed from its start state), each with the
    # particles uploaded before and downloaded after
    sim.set_timing(False)
    n = sim.num_particles()
    host_in = torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy()
    host_out = torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy()
    e2e_steps = args.steps
    sim.step(fsg.STEP_PICFLIP, sc.dt)  # graph for this configuration
    sim.restore(start)
    start.close()
    host_in[:] = sim.particles()
    sim.synchronize()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.set_particles(host_in)
        sim.step(fsg.STEP_PICFLIP, sc.dt)
        sim.lib.fs_get_particles(sim.h, host_out.ctypes.data, n)
        host_in, host_out = host_out, host_in
    sim.synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, "cuda:%d" % local_rank)
    e2e_value = sc.cells * e2e_steps * world / t_e2e

    if rank != 0:
        return
    sim.close()
    peak, peak_kind = peaks()
    forms = None
    if world == 1 and not args.no_forms:
        forms = {"batched": measure_batched(args, local_rank, value, flush),
                 "multigrid": measure_multigrid(args, local_rank, value, flush),
                 "large_step": measure_large_step(args, local_rank, flush),
                 "mixed_precision": measure_projection(args, local_rank)}
        if args.trajectory_steps > 0:
            forms["trajectory_500"] = measure_trajectory(args, local_rank, flush, peak)
        if args.phases_size > 0:
            forms["phases_4096"] = measure_phases(args, local_rank, flush, peak)
        if args.smoke_size > 0:
            forms["smoke"] = measure_smoke(args, local_rank)
    # roofline of the dominant kernel (the CG)
    cg_s = sum(cg_ms) / 1000.0
    achieved = CG_BYTES_PER_CELL_ITER * fi / cg_s / 1e9 if cg_s > 0 else None
    traffic = read_traffic()
    # CPU baseline: the oracle on the state at the start of the timed region
    kind = cpu_oracle_kind()
    if args.no_cpu:
        ctimes = [float("nan")]
    else:
        o = cpu_sim_from_state(sc, kind, grids0, parts0)
        ctimes = time_cpu_steps(o, sc, 1, args.cpu_budget)
    cpu_value = sc.cells * len(ctimes) / sum(ctimes)
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 dam break)",
        "config": config_of(sc),
        "measurement": {"parallelism": "replicas" if world > 1 else "single GPU",
                        "l2": "256 MiB written before every timed step; the step's CUDA events exclude it",
                        "timed_steps": "steps %d..%d of the workload (W warm-up steps first, the last of them "
                                       "recording the timed graph)" % (args.warmup + 1, args.warmup + args.steps),
                        "cg_iterations_mean": float(np.mean(iters)), "cg_iterations": iters},
        "phases_ms_per_step": {k: v / args.steps for k, v in phases.items()},
        "gpu_launches": int(launches),
        "e2e": {"value": e2e_value, "unit": UNIT, "steps": e2e_steps,
                "h2d_bytes_per_step": int(n * 16), "d2h_bytes_per_step": int(n * 16),
                "path": "fs_set_particles (pinned host) + fs_step + fs_get_particles (pinned host)"},
        "roofline": {"kernel": "k_cg (persistent Jacobi-PCG)", "bound": "hbm", "achieved": achieved,
                     "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "algorithmic_bytes": "%d B per fluid cell per CG iteration x sum(F x I) = %d B"
                                          % (CG_BYTES_PER_CELL_ITER, CG_BYTES_PER_CELL_ITER * fi),
                     "cg_ms_per_step": 1000.0 * cg_s / args.steps,
                     "per_phase": per_phase_rows(bsum, phases, args.steps, peak), "per_phase_model": PHASE_MODEL},
        "cpu_baseline": {"value": cpu_value, "unit": UNIT, "cores": 1, "host_cores": os.cpu_count(),
                         "kind": "reference" if kind == "reference" else "port",
                         "sample": "1 stepPICFLIP of the same workload from the GPU state at the start of "
                                   "the timed region (%.1f s), single thread" % sum(ctimes)},
        "clocks": clocks,
    }
    if forms:
        line["forms"] = forms
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    try:
        if args.impl == "reference":
            run_reference(args, rank)
        else:
            run_gpu(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
