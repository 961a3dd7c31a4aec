#!/usr/bin/env python
"""Throughput of the CABARET channel time step on GB300 (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: the FP64 channel at 256x128x128 cells, Re_b 5600, c = 10, CFL 0.2, bulk forcing,
seeded perturbations (the reference-parity configuration).  One "step" is one full time
step (main.cpp:82-91).  Metric: Mcell-steps/s = cells * steps / seconds.  The FP32 path at
512x256x256 is measured beside it (key "fp32"), and so is a batched ensemble of 64
independent FP32 channels of mixed sizes (key "ensemble").  Synthetic data: the seeded channel state
is the benchmark input (the reference has no dataset).

--impl reference times the reference's CPU step on the host cores instead: its C restatement
(oracle/ark_oracle.c, bit-identical to the reference on every pinned case), with all host
threads.  The reference compiled in place (oracle/_ref) cannot stand in here: its sources are
not part of this repository, so it exists only where the reference checkout does.

Under torchrun (N > 1) every rank advances its own independent channel (replicas; the
path has no exchange on one GPU per rank), timed between barriers; value = all ranks'
cell-steps / max rank time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ark-cpp-mpi_gb300"))
sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s on 1 GB300, FP32 vs plain FP64 at stated error; % HBM roofline"
UNIT = "Mcell-steps/s"

# Algorithmic (compulsory) values moved per cell by each launch of the fused step: every
# input element read once, every output element written once (faces counted once per cell:
# each face is shared by two cells).  Flags are 1 byte per cell.
ALGO_VALUES = {
    "finalize_dt": (0, 0),
    "wrap_con": (0, 0),
    "phase1_stress_forces": (26, 1),  # Con 4 + faces 15 -> nCon 4 + f 3
    "wrap_phase2": (0, 0),
    "sweep_x1": (17, 1),              # Con 4 + nCon 4 + faces 4 -> faces 5
    "sweep_x2": (17, 1),
    "sweep_x3": (17, 1),
    "phase1_forces": (26, 1),         # Con 4 + faces 15 + f 3 -> nCon 4
}
# FP32 stores no face density (it is ro0 + p/c^2): three values fewer per Phase1 and one
# fewer per sweep.
ALGO_VALUES_FP32 = dict(ALGO_VALUES, phase1_stress_forces=(23, 1), phase1_forces=(23, 1), sweep_x1=(16, 1),
                        sweep_x2=(16, 1), sweep_x3=(16, 1),
                        # Phase2 and the second Phase1 in one kernel: Con 4 + nCon 4 + faces 12 + f 3
                        # -> faces 12 + new level 4
                        phase2_phase1_forces=(39, 1),
                        # Phase1 + stress with the x1 sweep folded in: its 23 values plus the 4 new
                        # x faces (and the 4 new z faces with the x3 sweep too)
                        phase1_stress_sweep_x1=(27, 1), phase1_stress_sweep_x1_x3=(31, 1),
                        phase1_stress_sweep_x3=(27, 1))
# Persistent state per cell: cell rho,u1,u2,u3 + 3 face sets x {p,u1,u2,u3}; read and
# written once per step (the step's algorithmic bytes).
STEP_VALUES = 2 * 16


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_cell():
    """DRAM bytes per cell of each kernel from the committed ncu summary (or {})."""
    path = os.path.join(ROOT, "profiles", "traffic_per_cell.txt")
    out = {}
    if os.path.isfile(path):
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 3 and not line.startswith("#"):
                    out[(parts[0], parts[1])] = float(parts[2])
    return out


def ncu_fp64_pipe():
    """FP64 pipe activity (fraction of its peak) of each FP64 kernel from the committed ncu
    summary (or {})."""
    path = os.path.join(ROOT, "profiles", "fp64_pipe_per_kernel.txt")
    out = {}
    if os.path.isfile(path):
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 3 and not line.startswith("#"):
                    out[(parts[0], parts[1])] = float(parts[2]) / 100.0
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 25 ms while running (a 20-step FP64 region lasts about 70 ms)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join("/tmp", f"ark_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "-i", str(self.device),
                                          "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.isfile(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        with open(self.path) as f:
            for line in f:
                v = [x.strip() for x in line.split(",")]
                if len(v) < 9:
                    continue
                try:
                    sm.append(float(v[1]))
                    smax.append(float(v[2]))
                except ValueError:
                    continue
                for nm, flag in zip(names, v[5:9]):
                    if flag.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        return world, rank, local, dist
    return 1, 0, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


SEED = 1000  # seed of the channel state of rank 0 (rank r: SEED + r), both arms


def workload(C, re_b, precision):
    """The workload string both arms report for a grid (identical for identical work)."""
    return f"channel {C[0]}x{C[1]}x{C[2]} {precision.upper()} Re_b={re_b:g}, c=10, CFL 0.2, bulk forcing"


def channel_params(arkgpu, C, re_b, precision):
    return arkgpu.make_params(*C, re_b=re_b, sound=10.0, rho0=1.0, cfl=0.2, precision=precision)


def gpu_leg(arkgpu, C, re_b, precision, steps, warmup, device, seed, kernel_steps=10):
    """Device-timed throughput, per-launch times and the roofline of the dominant kernel."""
    p = channel_params(arkgpu, C, re_b, precision)
    p.device = device
    st = arkgpu.channel_init(p, seed=seed, amp=0.1)
    cells = C[0] * C[1] * C[2]
    with arkgpu.Context(p) as ctx:
        ctx.upload(st)
        shapes = ctx.autotune(10)  # the library's shape autotuner (10 steps per candidate: close
        # candidates differ by about 1%), then the same start state
        ctx.upload(st)
        del st
        ctx.step(warmup)
        ctx.sync()
        with ClockSampler(device) as clk:
            ms = ctx.time_steps(steps)
        clocks = clk.summary()
        ktimes = ctx.kernel_times(kernel_steps)
        sc = ctx.scalars()
    return {"cells": cells, "ms": ms, "clocks": clocks, "ktimes": ktimes, "dt": sc.dt, "ub": sc.bulk_velocity,
            "shapes": shapes}


def roofline(kt, cells, word, peak, peak_kind, traffic_tab, prec_name):
    name, ms = max(kt, key=lambda x: x[1])
    vals, flag_b = (ALGO_VALUES_FP32 if word == 4 else ALGO_VALUES).get(name, (0, 0))
    algo = cells * (vals * word + flag_b)
    achieved = algo / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
    tpc = traffic_tab.get((prec_name, name))
    r = {"kernel": name, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
         "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
         "traffic": (round(tpc * cells) if tpc is not None else None),
         "algorithmic_bytes": algo, "launch_ms": round(ms, 4)}
    pipe = ncu_fp64_pipe().get((prec_name, name)) if prec_name == "fp64" else None
    if pipe is not None:
        # the FP64 kernels issue FP64 arithmetic at the pipe's limit; HBM is far from it
        r["fp64_pipe"] = {"active_frac": pipe, "source": "ncu sm__pipe_fp64_cycles_active (profiles)",
                          "note": "bound by FP64 issue (GB300 FP64 is about 1.2 TFLOP/s), not by HBM"}
    return r


def e2e_leg(arkgpu, C, re_b, precision, steps, device, seed, roundtrip=True):
    """Through the C ABI with host buffers, as a program replacing the reference's main loop
    uses it: upload the whole state from pinned host memory, then every step run ark_step and
    read the step's scalars back (dt, TIME, bulk velocity: a synchronous device->host read),
    then download the whole state.  All of it is inside the timed region."""
    p = channel_params(arkgpu, C, re_b, precision)
    p.device = device
    st = arkgpu.channel_init(p, seed=seed, amp=0.1)
    hs = arkgpu.PinnedState(p)
    hs.fill(st)
    del st
    cells = C[0] * C[1] * C[2]
    with arkgpu.Context(p) as ctx:
        ctx.upload_struct(hs.struct(True))
        ctx.autotune(10)  # kernel shapes, before anything is timed
        ctx.upload_struct(hs.struct(True))  # warm-up: graphs, first transfers
        ctx.step(2)
        ctx.scalars()
        ctx.download_struct(hs.struct(False))
        t0 = time.perf_counter()
        ctx.upload_struct(hs.struct(True))
        for _ in range(steps):
            ctx.step(1)
            ctx.scalars()
        ctx.download_struct(hs.struct(False))
        secs = time.perf_counter() - t0
        ctx.sync()
        rt = None
        if roundtrip:
            rt = full_state_roundtrip(ctx, hs, cells, steps)
    up = hs.nbytes(True)
    down = hs.nbytes(False)
    scal = 5 * 8  # the ark_scalars read every step
    hs.close()
    out = {"value": round(cells * steps / secs / 1e6, 3), "unit": UNIT,
           "h2d_bytes_per_step": round(up / steps), "d2h_bytes_per_step": round(down / steps) + scal,
           "steps": steps, "precision": "fp64" if precision == arkgpu.FP64 else "fp32", "grid": list(C),
           "note": "one job: state upload, steps each with a synchronous scalar read-back, state download"}
    if rt is not None:
        out["state_roundtrip_every_step"] = rt
    return out


def full_state_roundtrip(ctx, hs, cells, steps):
    """The whole state uploaded, stepped once and downloaded, every step (a caller that keeps
    the state on the host between steps)."""
    h = hs.struct(False)
    ctx.upload_struct(h)
    ctx.step(1)
    ctx.download_struct(h)
    n_rt = max(3, steps // 10)
    t1 = time.perf_counter()
    for _ in range(n_rt):
        ctx.upload_struct(h)
        ctx.step(1)
        ctx.download_struct(h)
    rt_secs = time.perf_counter() - t1
    down = hs.nbytes(False)
    return {"value": round(cells * n_rt / rt_secs / 1e6, 3), "unit": UNIT, "h2d_bytes_per_step": down,
            "d2h_bytes_per_step": down, "steps": n_rt}


def fp32_error_report():
    """The committed FP32-vs-FP64 error report of the 512x256x256 channel after 2000 steps
    (ark-cpp-mpi_gb300/precision_report.py, profiles/fp32_error_512x256x256_2000_steps.json),
    or None."""
    path = os.path.join(ROOT, "profiles", "fp32_error_512x256x256_2000_steps.json")
    if not os.path.isfile(path):
        return None
    with open(path) as f:
        d = json.load(f)
    return {"grid": d["grid"], "steps": d["steps"], "re_b": d["re_b"], **d["errors"],
            "source": "profiles/fp32_error_512x256x256_2000_steps.json (precision_report.py on the GPU)"}


ENSEMBLE_GRIDS = ((32, 32, 32), (64, 32, 32), (64, 48, 48), (96, 64, 64), (128, 64, 64))


def ensemble_leg(arkgpu, members, steps, warmup, device, seed=4242, shape=None):
    """A batched ensemble of independent FP32 channels: grids drawn from ENSEMBLE_GRIDS, Re_b
    uniform in [2000, 6000], perturbation amplitude uniform in [0.05, 0.15], bulk forcing;
    one persistent launch per phase under a CUDA graph, kernel shapes autotuned first (or set
    to `shape`: Phase1 + stress shape, second Phase1 shape, segment)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    params, states = [], []
    for q in range(members):
        C = ENSEMBLE_GRIDS[int(rng.integers(len(ENSEMBLE_GRIDS)))]
        p = channel_params(arkgpu, C, float(rng.uniform(2000.0, 6000.0)), arkgpu.FP32)
        p.device = device
        params.append(p)
        states.append((C, float(rng.uniform(0.05, 0.15))))
    cells = sum(C[0] * C[1] * C[2] for C, _ in states)
    with arkgpu.Ensemble(params) as E:
        for q, (p, (C, amp)) in enumerate(zip(params, states)):
            E.upload(q, arkgpu.channel_init(p, seed=seed + q, amp=amp))
        t0 = time.perf_counter()
        if shape:
            E.set_shape(*shape)
            shape = {"march_phase1_stress": shape[0], "march_phase1": shape[1], "segment": shape[2], "us_per_step": None}
        else:
            shape = E.autotune(3)
        tune_s = time.perf_counter() - t0
        E.step(warmup)
        E.sync()
        with ClockSampler(device) as clk:
            ms = E.time_steps(steps)
        clocks = clk.summary()
        ktimes = E.kernel_times(5)
        finite = all(math.isfinite(E.scalars(q).dt) for q in range(members))
    step_s = ms * 1e-3 / steps
    counts = {f"{a}x{b}x{c}": sum(1 for C, _ in states if C == (a, b, c)) for a, b, c in ENSEMBLE_GRIDS}
    return {"value": round(cells * steps / (ms * 1e-3) / 1e6, 3), "unit": UNIT, "members": members,
            "cells": cells, "grids": counts, "steps": steps, "ms_per_step": round(ms / steps, 4),
            "dtype": "f32 (f64 reductions)", "launches_per_step": len(ktimes), "autotuned_shape": shape,
            "autotune_s": round(tune_s, 3), "finite": finite,
            "kernels_ms": {k: round(v, 4) for k, v in ktimes}, "ktimes": ktimes,
            "step_roofline": {"bytes_per_cell": STEP_VALUES * 4,
                              "achieved": round(cells * STEP_VALUES * 4 / step_s / 1e9, 1), "unit": "GB/s"},
            "clocks": clocks}


def cpu_sample(C, re_b, threads, budget_s, max_steps=400):
    """Full steps of the oracle's C restatement of the reference step on `threads` host
    threads, for about budget_s seconds: (Mcell-steps/s, steps, seconds)."""
    import oracle

    oracle.build(port=True, ref=False)
    p = oracle.channel_params(*C, re_b=re_b, seed=SEED)
    o = oracle.Port(p, threads=threads)
    o.load(oracle.channel_state(p))
    o.run(1)  # warm-up
    n, t0 = 0, time.perf_counter()
    while n < max_steps and time.perf_counter() - t0 < budget_s:
        o.run(1)
        n += 1
    secs = time.perf_counter() - t0
    return C[0] * C[1] * C[2] * n / secs / 1e6, n, secs


def cpu_leg(C, re_b, budget_s=12.0):
    """The oracle's C restatement of the reference step on all host cores, and on one."""
    threads = os.cpu_count() or 1
    v, n, secs = cpu_sample(C, re_b, threads, budget_s)
    v1, n1, secs1 = cpu_sample(C, re_b, 1, budget_s)
    return {"value": round(v, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} full steps of the {workload(C, re_b, 'fp64')}, {threads} OpenMP threads ({secs:.1f} s)",
            "one_core": {"value": round(v1, 4), "unit": UNIT, "cores": 1,
                         "sample": f"{n1} full steps, 1 thread ({secs1:.1f} s)"}}


def reference_arm(args, world, rank, dist):
    """--impl reference: the reference's CPU step (C restatement) timed on the host cores."""
    if rank != 0:
        return 0
    import oracle

    oracle.build(port=True, ref=False)
    threads = os.cpu_count() or 1
    C = tuple(args.grid)
    p = oracle.channel_params(*C, re_b=args.re, seed=SEED)
    o = oracle.Port(p, threads=threads)
    o.load(oracle.channel_state(p))
    tw = time.perf_counter()
    o.run(args.warmup)
    per_step = (time.perf_counter() - tw) / max(1, args.warmup)
    # a bounded sample: at most about 90 s of timed CPU work, whatever --steps asks
    steps = max(1, min(args.steps, int(90.0 / max(per_step, 1e-9))))
    t0 = time.perf_counter()
    o.run(steps)
    secs = time.perf_counter() - t0
    cells = C[0] * C[1] * C[2]
    v = cells * steps / secs / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": UNIT, "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": round(secs * 1e3 / steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded channel state)",
            "config": {"workload": workload(C, args.re, "fp64"), "grid": list(C), "precision": "fp64",
                       "seed": SEED, "parallelism": "host threads"},
            "cpu_baseline": {"value": round(v, 4), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{steps} full steps of the {C[0]}x{C[1]}x{C[2]} channel "
                                       f"({args.steps} asked), {threads} OpenMP threads"},
            "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--grid", type=int, nargs=3, default=(256, 128, 128))
    ap.add_argument("--re", type=float, default=5600.0)
    ap.add_argument("--fp32-grid", type=int, nargs=3, default=(512, 256, 256))
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--ensemble", type=int, default=64, help="ensemble members (0: no ensemble leg)")
    ap.add_argument("--ensemble-steps", type=int, default=500)
    ap.add_argument("--ensemble-shape", type=int, nargs=3, default=None,
                    help="fixed ensemble kernel shape (Phase1 + stress, second Phase1, segment) instead of autotuning")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        rc = reference_arm(args, world, rank, dist)
        if dist is not None:
            dist.destroy_process_group()
        return rc

    import arkgpu

    arkgpu.lib()
    device = local
    C = tuple(args.grid)
    peak, peak_kind = measured_peaks()
    traffic = ncu_traffic_per_cell()

    barrier(dist)
    g = gpu_leg(arkgpu, C, args.re, arkgpu.FP64, args.steps, args.warmup, device, seed=SEED + rank)
    barrier(dist)
    ms = max_over_ranks(dist, g["ms"])
    total_cells = g["cells"] * world
    value = total_cells * args.steps / (ms * 1e-3) / 1e6
    launches_per_step = len(g["ktimes"])

    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded channel state)",
            "config": {"workload": workload(C, args.re, "fp64"), "grid": list(C), "precision": "fp64", "seed": SEED,
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": f"inputs larger than L2: {g['cells'] * 8 * 41 / 1e9:.2f} GB of state streamed per step"},
            "clocks": g["clocks"], "kernel_shapes": g["shapes"],
            "gpu_launches": launches_per_step * args.steps}
    line["roofline"] = roofline(g["ktimes"], g["cells"], 8, peak, peak_kind, traffic, "fp64")
    step_s = ms * 1e-3 / args.steps
    line["step_roofline"] = {"bytes_per_cell": STEP_VALUES * 8,
                             "achieved": round(g["cells"] * STEP_VALUES * 8 / step_s / 1e9, 1),
                             "peak": peak, "unit": "GB/s",
                             "frac": round(g["cells"] * STEP_VALUES * 8 / step_s / 1e9 / peak, 4)}
    line["kernels_ms"] = {k: round(v, 4) for k, v in g["ktimes"]}

    if rank == 0 and not args.no_fp32:
        C32 = tuple(args.fp32_grid)
        f = gpu_leg(arkgpu, C32, args.re, arkgpu.FP32, max(20, args.steps // 3), args.warmup, device, seed=77)
        f_steps = max(20, args.steps // 3)
        fv = f["cells"] * f_steps / (f["ms"] * 1e-3) / 1e6
        f_step_s = f["ms"] * 1e-3 / f_steps
        line["fp32"] = {"value": round(fv, 3), "unit": UNIT, "grid": list(C32), "steps": f_steps,
                        "ms_per_step": round(f["ms"] / f_steps, 4), "dtype": "f32 (f64 reductions)",
                        "roofline": roofline(f["ktimes"], f["cells"], 4, peak, peak_kind, traffic, "fp32"),
                        "step_roofline": {"bytes_per_cell": STEP_VALUES * 4,
                                          "achieved": round(f["cells"] * STEP_VALUES * 4 / f_step_s / 1e9, 1),
                                          "peak": peak, "unit": "GB/s",
                                          "frac": round(f["cells"] * STEP_VALUES * 4 / f_step_s / 1e9 / peak, 4)},
                        "kernels_ms": {k: round(v, 4) for k, v in f["ktimes"]}, "clocks": f["clocks"],
                        "kernel_shapes": f["shapes"], "error": fp32_error_report()}
        line["gpu_launches"] += len(f["ktimes"]) * f_steps

    if rank == 0 and args.ensemble > 0:
        e = ensemble_leg(arkgpu, args.ensemble, args.ensemble_steps, args.warmup, device, shape=args.ensemble_shape)
        e["step_roofline"].update(peak=peak, frac=round(e["step_roofline"]["achieved"] / peak, 4))
        e["roofline"] = roofline(e.pop("ktimes"), e["cells"], 4, peak, peak_kind, traffic, "ensemble")
        line["ensemble"] = e
        line["gpu_launches"] += e["launches_per_step"] * args.ensemble_steps

    if rank == 0:
        line["e2e"] = e2e_leg(arkgpu, C, args.re, arkgpu.FP64, args.e2e_steps, device, seed=SEED)
        if "fp32" in line:
            line["fp32"]["e2e"] = e2e_leg(arkgpu, tuple(args.fp32_grid), args.re, arkgpu.FP32, args.e2e_steps,
                                          device, seed=77, roundtrip=False)
        if world == 1 and not args.no_cpu:
            line["cpu_baseline"] = cpu_leg(C, args.re)
        print(json.dumps(line), flush=True)
    barrier(dist)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
