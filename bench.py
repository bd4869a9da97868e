#!/usr/bin/env python
"""Benchmark of the fused WENO5 / Lax-Friedrichs / RK3 stage path on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: 1D inviscid Burgers on 2^24 uniform cells of [-5, 5], u0 a seeded sum of 8
Gaussians, WENO5 (k = 3, eps = 1e-6), global Lax-Friedrichs flux with alpha = max|u0|, copy
boundaries, rktvd order 3, CFL 0.4.  One step is one RK3 time step over the whole line
(three fused stage kernels); the metric is cell-updates per second, one cell-update being
one cell advanced one full RK3 step.

The headline line (printed last) is the MIXED numerics mode: the FP64 state and stage combines
with the right-hand side evaluated in difference form on the FP32 pipe, parity-tested against
the oracle at the same 1e-12 bar as the plain FAST FP64 path.  Every other form of the metric
is printed first, one short JSON line each ("form": name; values in cell-updates/s unless a
key says otherwise; hbm_frac from the algorithmic bytes per cell-update of the form):
the plain FP64 path and the compensated FP32 form of the same line, the line with WENO3, the
2D grids, the batched lines, the adjoint and the reference's own 500-cell driver loop.

`value` times K steps on device-resident data with CUDA events on the library's stream.
`e2e` times K calls of the reference-facing integrate(u, t, tout, dt, itask=2) with u in
pinned host memory: each call copies u to the device, takes one step and copies u back.
`--impl reference` times the CPU restatement of the reference (oracle/, its -O3 build, all
host threads) on the same workload.

Under torchrun (N > 1) every rank integrates its own replica of the line (replicas only:
the single-line path has no exchange step here); value = all ranks' cell-updates / the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for p in (ROOT, ROOT / "hr-weno_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

METRIC = "WENO5-RK3 cell-updates/s & HBM-roofline %; batched/FP32/adjoint vs plain FP64"
UNIT = "cell-updates/s"
NC = 1 << 24
# algorithmic HBM bytes of one FP64 RK3 cell-update: stage 1 reads u, writes u1 (16 B);
# stage 2 reads u, u1, writes u2 (24 B); stage 3 reads u, u2, writes u (24 B)
BYTES_PER_CELL_UPDATE = 64
LAUNCHES_PER_STEP = 3
# compensated FP32, algorithmic bytes of a state u = hi + lo and one float per increment:
# 40 B per RK3 cell-update (the lo word of u read and written in the last stage beside the
# 32 B of a plain FP32 RK3 step).  The kernel moves 48 B: stage 1 reads hi, lo and writes d1
# (12 B); stage 2 reads hi, lo, d1 and writes d2 (16 B); stage 3 reads hi, lo, d2 and writes
# hi, lo (20 B).
F32C_BYTES_PER_CELL_UPDATE = 40
F32C_MOVED_BYTES_PER_CELL_UPDATE = 48
# REAL32 (a REAL32 build of the reference, FP32 state): 32 B per RK3 cell-update, half of FP64's
F32_BYTES_PER_CELL_UPDATE = 32
L2_BYTES = 126 * 1024 * 1024

# DRAM bytes per cell and stage launch of the MIXED stage kernel, measured by ncu on the
# 2^24-cell line (dram__bytes_read.sum + dram__bytes_write.sum of the three RK3 stage launches
# of one step, divided by cells x 3); profiles/stage1d_mixed_weno5_rk3.md.
NCU_DRAM_BYTES_PER_CELL_LAUNCH = 969.9e6 / (3 * (1 << 24))


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


# ------------------------------------------------------------------------------------------
# clocks during the timed region
# ------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = []
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        reasons = set()
        for _, _, flags in rows:
            for name, flag in zip(self.NAMES, flags):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows), "samples": len(rows),
                "reasons": sorted(reasons)}


# ------------------------------------------------------------------------------------------
# distributed plumbing (replicas)
# ------------------------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg is not None:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if self.pg is None:
            return x
        import torch
        dev = "cuda" if torch.cuda.is_available() else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg is not None:
            self.pg.destroy_process_group()


# ------------------------------------------------------------------------------------------
# CPU: the oracle (restatement of the reference), bounded sample
# ------------------------------------------------------------------------------------------
def cpu_rate(u0: np.ndarray, prob, dt: float, steps: int, threads: int):
    """cell-updates/s of the oracle over `steps` RK3 steps of the full line."""
    from oracle import oracle
    oracle.select_build("baseline")
    used = oracle.set_threads(threads)
    ode = oracle.ODE(prob, u0.size, 0, 3)
    u = u0.copy()
    t0 = time.perf_counter()
    ode.integrate(u, 0.0, (steps - 0.5) * dt, dt)
    el = time.perf_counter() - t0
    assert ode.info()[2] == steps
    return u0.size * steps / el, el, used


def run_reference(args) -> None:
    from hrweno import workloads
    prob, u0, dt = workloads.large_burgers(NC, k=3)
    threads = os.cpu_count() or 1
    # warm-up (page-in, thread pool), then K steps each timed as one bounded sample
    _, el1, used = cpu_rate(u0, prob, dt, 1, threads)
    for _ in range(max(args.warmup - 1, 0)):
        cpu_rate(u0, prob, dt, 1, threads)
    # keep the run to a few minutes: cells of each step's sample scale down if needed
    budget_s = 150.0
    n = NC
    while n > (1 << 16) and el1 * (n / NC) * args.steps > budget_s:
        n //= 2
    if n != NC:
        prob, u0s, dt = workloads.large_burgers(n, k=3, u0=u0[:: NC // n].copy())
    else:
        u0s = u0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_rate(u0s, prob, dt, 1, threads)
    el = time.perf_counter() - t0
    v = n * args.steps / el
    sample = (f"{args.steps} RK3 steps, each one step over {n} cells"
              + (" (a strided sub-line of the 2^24-cell line)" if n != NC else " (the full line)")
              + ", oracle restatement -O3")
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded 8-Gaussian u0 (numpy default_rng(1))",
        "config": config_dict(), "impl": "reference",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": used, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_dict() -> dict:
    mib = NC * 8 >> 20
    name = "2^24" if NC == 1 << 24 else str(NC)
    return {"workload": f"burgers1d_{name}_weno5_lf_rk3", "cells": NC, "k": 3, "eps": 1e-6,
            "flux": "lax_friedrichs", "alpha": "max|u0|", "bc": "copy", "cfl": 0.4,
            "integrator": "rktvd order 3",
            "numerics": "mixed: FP64 state; RHS in float-pair difference form on the FP32 pipe",
            "l2": (f"inputs larger than L2: u, d1, d2 are {mib} MiB each ({3 * mib} MiB working set)"
                   if 3 * NC * 8 > 126 << 20 else
                   f"L2-resident: u, d1, d2 are {NC * 8 >> 10} KiB each (a reduced line, not the benchmark workload)")}


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------
def time_line(prob, u0, dt, dtype, args, dist, stream, clk=None):
    """(seconds for K RK3 steps after W untimed ones, the state, the handle) on device memory"""
    import torch

    import hrweno
    ode = hrweno.rktvd(prob, u0.size, 3, dtype=dtype)
    ode.set_stream(stream.cuda_stream)
    u = torch.from_numpy(u0).cuda()
    t = ode.integrate(u, 0.0, (args.warmup - 0.5) * dt, dt)
    torch.cuda.synchronize()
    n0 = ode.nsteps
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    if clk is not None:
        clk.__enter__()
    e0.record(stream)
    t = ode.integrate(u, t, t + (args.steps - 0.5) * dt, dt)
    e1.record(stream)
    torch.cuda.synchronize()
    if clk is not None:
        clk.__exit__(None, None, None)
    dist.barrier()
    assert ode.nsteps - n0 == args.steps, (ode.nsteps - n0, args.steps)
    assert bool(torch.isfinite(u).all())
    return dist.max(e0.elapsed_time(e1) * 1e-3), u, ode


def hbm(bytes_per_cell_update: float, value: float, dist) -> float:
    return bytes_per_cell_update * value / dist.world / 1e9 / peaks()["hbm_gbs"]


LINE_FORMS = (("fast", "f64"), ("mixed", "f64"), ("fast", "f32c"), ("strict", "f32"))


def run_line_forms(args, dist: Dist, k: int, u_ref=None) -> list:
    """Short lines for the plain FP64 (FAST), MIXED (k = 2 only; k = 3 is the headline),
    compensated FP32 and REAL32 forms of the 2^24-cell line with WENO(2k-1)."""
    import torch

    from hrweno import workloads

    stream = torch.cuda.Stream()
    out = []
    res = {}
    for num, dtype in LINE_FORMS:
        if k == 3 and num == "mixed":
            continue
        prob, u0, dt = workloads.large_burgers(NC, k=k, numerics=num)
        if dtype == "f32":
            u0 = u0.astype(np.float32)
        el, u, _ = time_line(prob, u0, dt, dtype, args, dist, stream)
        v = dist.world * NC * args.steps / el
        res[(num, dtype)] = u
        name = f"1d_k{k}_{dtype if dtype != 'f64' else num}"
        line = {"form": name, "value": v, "ms": 1e3 * el / args.steps}
        if dtype == "f32c":
            line["hbm_frac"] = hbm(F32C_BYTES_PER_CELL_UPDATE, v, dist)
            line["moved_B"] = F32C_MOVED_BYTES_PER_CELL_UPDATE
        elif dtype == "f32":
            line["hbm_frac"] = hbm(F32_BYTES_PER_CELL_UPDATE, v, dist)
        else:
            line["hbm_frac"] = hbm(BYTES_PER_CELL_UPDATE, v, dist)
        out.append(line)
    base = u_ref if u_ref is not None else res[("mixed", "f64")]
    for line, key in zip(out, [kk for kk in LINE_FORMS if kk in res]):
        if key != ("mixed", "f64") or u_ref is not None:
            d = (res[key] - base).abs()
            line["l1_vs_mixed"] = float(d.sum() / base.abs().sum())
    return out


def run_ours(args, dist: Dist):
    """(headline line, form lines): the MIXED form of the 2^24-cell WENO5 line."""
    import torch

    import hrweno
    from hrweno import workloads

    dev = dist.local if dist.world > 1 else 0
    torch.cuda.set_device(dev)
    prob, u0, dt = workloads.large_burgers(NC, k=3, numerics="mixed")
    stream = torch.cuda.Stream()

    # ---- device-resident K steps ---------------------------------------------------------
    clk = ClockSampler(dev)
    el, u, ode = time_line(prob, u0, dt, "f64", args, dist, stream, clk=clk)
    value = dist.world * NC * args.steps / el
    forms = run_line_forms(args, dist, 3, u_ref=u) if "line" in args.forms else []

    # ---- e2e: reference-facing call on pinned host memory, one step per call -------------
    ode2 = hrweno.rktvd(prob, NC, 3)
    ode2.set_stream(stream.cuda_stream)
    uh = torch.from_numpy(u0.copy()).pin_memory()
    th = 0.0
    for _ in range(max(1, min(args.warmup, 3))):
        th = ode2.integrate(uh, th, th + 0.5 * dt, dt, itask=2)
    dist.barrier()
    torch.cuda.synchronize()
    h0 = time.perf_counter()
    for _ in range(args.steps):
        th = ode2.integrate(uh, th, th + 0.5 * dt, dt, itask=2)
    torch.cuda.synchronize()
    e2e_el = dist.max(time.perf_counter() - h0)
    dist.barrier()
    e2e = {"value": dist.world * NC * args.steps / e2e_el, "unit": UNIT,
           "h2d_bytes_per_step": 8 * NC, "d2h_bytes_per_step": 8 * NC}

    if dist.rank != 0:
        return None, forms

    pk = peaks()
    launches = args.steps * LAUNCHES_PER_STEP
    launch_s = el / launches
    bytes_per_launch = BYTES_PER_CELL_UPDATE * NC / LAUNCHES_PER_STEP
    achieved = bytes_per_launch / launch_s / 1e9
    traffic = (None if NCU_DRAM_BYTES_PER_CELL_LAUNCH is None
               else NCU_DRAM_BYTES_PER_CELL_LAUNCH * NC)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                "peak_src": "measured (MEASURED_PEAKS.json hbm_gbs)" if pk["src"] == "measured"
                else "fallback 6.8 TB/s"}

    # ---- CPU baseline: the oracle's -O3 build, 1 core, bounded sample ---------------------
    cpu = None
    if not args.no_cpu:
        steps = 3
        v, el_cpu, used = cpu_rate(u0, prob, dt, steps, 1)
        cpu = {"value": v, "unit": UNIT, "cores": used, "kind": "port",
               "sample": f"{steps} RK3 steps of the full 2^24-cell line ({el_cpu:.1f} s), oracle "
                         f"restatement -O3, 1 thread; host has {os.cpu_count()} cores"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded 8-Gaussian u0 (numpy default_rng(1))",
        "config": config_dict(),
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches + 1,  # 3 stage kernels per step and one max|u| reduction
        "clocks": clk.summary(),
    }
    return line, forms


# ------------------------------------------------------------------------------------------
# 2D population balance (example2): 4096^2, WENO5 dimension by dimension, upwind Godunov,
# mstvd; one step is one multistep update of the grid (one fused launch)
# ------------------------------------------------------------------------------------------
PBE_N = 4096
# mstvd FP64: read u^n, u^{n-4}, L^{n-4}; write u^{n+1}, L^n
PBE_BYTES_PER_CELL_UPDATE = 40


def pbe_config_dict(n: int) -> dict:
    return {"workload": f"pbe2d_{n}^2_weno5_godunov_mstvd", "cells": n * n, "k": 3,
            "eps": 1e-6, "flux": "godunov (upwind, g1 = 1 + 0.5 x1, g2 = 0.5)",
            "bc": "zero_inflow", "cfl": 0.4, "integrator": "mstvd (5-step, 3rd order)",
            "numerics": "fast",
            "l2": (f"inputs larger than L2: 5 + 4 ring slots of {n * n * 8 >> 20} MiB"
                   if 9 * n * n * 8 > 126 << 20 else
                   f"L2-resident: 5 + 4 ring slots of {n * n * 8 >> 20} MiB fit the 126 MiB L2 "
                   "(a secondary line; the 4096^2 grid is the L2-exceeding one)")}


def run_pbe2d(args, dist: Dist) -> dict | None:
    import torch

    import hrweno
    from hrweno import workloads

    dev = dist.local if dist.world > 1 else 0
    torch.cuda.set_device(dev)
    n = args.pbe_n
    cells = n * n
    prob, n0, dt = workloads.pbe_config(n, n)
    stream = torch.cuda.Stream()
    ode = hrweno.mstvd(prob, cells)
    ode.set_stream(stream.cuda_stream)
    u = torch.from_numpy(n0).cuda()
    # the RK3 start (4 steps + 4 right-hand sides) and W multistep steps, untimed
    t = ode.integrate(u, 0.0, (4 + args.warmup - 0.5) * dt, dt)
    torch.cuda.synchronize()
    n0steps = ode.nsteps
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    with ClockSampler(dev) as clk:
        e0.record(stream)
        t = ode.integrate(u, t, t + (args.steps - 0.5) * dt, dt)
        e1.record(stream)
        torch.cuda.synchronize()
    steps_done = ode.nsteps - n0steps
    assert steps_done == args.steps
    el = dist.max(e0.elapsed_time(e1) * 1e-3)
    value = dist.world * cells * args.steps / el
    # compensated FP32 on the same grid and steps, error against the FP64 result
    forms = {}
    if "line" in args.forms or "pbe2d" in args.forms:
        ode32 = hrweno.mstvd(prob, cells, dtype="f32c")
        ode32.set_stream(stream.cuda_stream)
        u32 = torch.from_numpy(n0).cuda()
        t32 = ode32.integrate(u32, 0.0, (4 + args.warmup - 0.5) * dt, dt)
        torch.cuda.synchronize()
        e0.record(stream)
        t32 = ode32.integrate(u32, t32, t32 + (args.steps - 0.5) * dt, dt)
        e1.record(stream)
        torch.cuda.synchronize()
        el32 = dist.max(e0.elapsed_time(e1) * 1e-3)
        diff = (u32 - u).abs()
        v32 = dist.world * cells * args.steps / el32
        # algorithmic bytes 28 B per multistep cell-update (the lo word of u read and written
        # beside the 20 B of plain FP32); the kernel moves 32 B (L(u^{n-4}) is a plain float)
        forms["f32c"] = {"value": v32, "unit": UNIT, "ms_per_step": 1e3 * el32 / args.steps,
                         "speedup_vs_f64": v32 / value, "bytes_per_cell_update": 28,
                         "moved_bytes_per_cell_update": 32,
                         "hbm_frac": 28 * v32 / dist.world / 1e9 / peaks()["hbm_gbs"],
                         "rel_l1_vs_f64": float(diff.sum() / u.abs().sum()),
                         "rel_linf_vs_f64": float(diff.max() / u.abs().max())}
        del ode32, u32, diff
        # accuracy at a stable step: 500 steps at CFL 0.3 on 1024^2 (at 0.4 the multistep
        # scheme is unstable here and any two implementations drift apart)
        m = 1024
        pa, na, dta = workloads.pbe_config(m, m, cfl=0.3)
        ua = torch.from_numpy(na.copy()).cuda()
        ub = torch.from_numpy(na.copy()).cuda()
        hrweno.mstvd(pa, m * m).integrate(ua, 0.0, 499.5 * dta, dta)
        hrweno.mstvd(pa, m * m, dtype="f32c").integrate(ub, 0.0, 499.5 * dta, dta)
        dd = (ua - ub).abs()
        forms["f32c"]["accuracy_1024_cfl0.3_500steps"] = {
            "rel_l1_vs_f64": float(dd.sum() / ua.abs().sum()),
            "rel_linf_vs_f64": float(dd.max() / ua.abs().max())}
        del ua, ub, dd
    # e2e: one multistep step per reference-facing call on pinned host memory
    ode2 = hrweno.mstvd(prob, cells)
    ode2.set_stream(stream.cuda_stream)
    uh = torch.from_numpy(n0.copy()).pin_memory()
    th = ode2.integrate(uh, 0.0, 4.5 * dt, dt)
    torch.cuda.synchronize()
    h0 = time.perf_counter()
    for _ in range(args.steps):
        th = ode2.integrate(uh, th, th + 0.5 * dt, dt)
    torch.cuda.synchronize()
    e2e_el = dist.max(time.perf_counter() - h0)
    if dist.rank != 0:
        return None
    pk = peaks()
    achieved = PBE_BYTES_PER_CELL_UPDATE * cells * args.steps / el / 1e9
    cpu = None
    if not args.no_cpu:
        from oracle import oracle
        oracle.select_build("baseline")
        m = 1024  # bounded sample: the 1024^2 grid, 3 multistep steps after the start
        p1, v1, dt1 = workloads.pbe_config(m, m)
        used = oracle.set_threads(1)
        o = oracle.ODE(p1, m * m, 1)
        tt = o.integrate(v1, 0.0, 4.5 * dt1, dt1)
        c0 = time.perf_counter()
        o.integrate(v1, tt, tt + 2.5 * dt1, dt1)
        cel = time.perf_counter() - c0
        cpu = {"value": m * m * 3 / cel, "unit": UNIT, "cores": used, "kind": "port",
               "sample": f"3 mstvd steps of the 1024^2 grid ({cel:.1f} s), oracle, 1 thread"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: Gaussian pulse at (0.2, 0.2), sigma 0.05",
        "config": pbe_config_dict(n),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": None,
                     "peak_src": pk["src"]},
        "cpu_baseline": cpu,
        "e2e": {"value": dist.world * cells * args.steps / e2e_el, "unit": UNIT,
                "h2d_bytes_per_step": 8 * cells, "d2h_bytes_per_step": 8 * cells},
        "forms": forms,
        "gpu_launches": steps_done,
        "clocks": clk.summary(),
    }
    return line


# ------------------------------------------------------------------------------------------
# batched: 4096 independent lines of log-uniform size in [64, 65536], half Burgers, half
# linear advection, k in {2, 3}, per-problem dt; one step advances every problem one RK3 step
# ------------------------------------------------------------------------------------------
BATCH_NPROB = 4096


def run_batched(args, dist: Dist) -> dict | None:
    import tempfile

    import torch

    import hrweno
    from hrweno import workloads

    dev = dist.local if dist.world > 1 else 0
    torch.cuda.set_device(dev)
    probs, lines, dts = workloads.batched_config(BATCH_NPROB, seed=7 + dist.rank)
    cells = int(sum(v.size for v in lines))
    stream = torch.cuda.Stream()
    b = hrweno.batch(probs, order=3)
    b.set_stream(stream.cuda_stream)
    packed = b.pack(lines)
    cache = str(Path(tempfile.gettempdir()) / "hrweno_batch_tune.txt")
    shapes = b.tune(packed, dts, probe_steps=3, cache_path=cache)
    u = torch.from_numpy(packed).cuda()
    t = np.zeros(BATCH_NPROB)
    b.advance(u, t, dts, args.warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    with ClockSampler(dev) as clk:
        e0.record(stream)
        b.advance(u, t, dts, args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    el = dist.max(e0.elapsed_time(e1) * 1e-3)
    value = dist.world * cells * args.steps / el
    assert bool(torch.isfinite(u).all())

    # the same batch in compensated FP32
    b32 = hrweno.batch(probs, order=3, dtype="f32c")
    b32.set_stream(stream.cuda_stream)
    shapes32 = b32.tune(packed, dts, probe_steps=3, cache_path=cache)
    u32 = torch.from_numpy(packed.copy()).cuda()
    t32 = np.zeros(BATCH_NPROB)
    b32.advance(u32, t32, dts, args.warmup)
    torch.cuda.synchronize()
    e0.record(stream)
    b32.advance(u32, t32, dts, args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    el32 = dist.max(e0.elapsed_time(e1) * 1e-3)
    d32 = (u32 - u).abs()
    f32c_form = {"value": dist.world * cells * args.steps / el32, "unit": UNIT,
                 "ms_per_step": 1e3 * el32 / args.steps, "shapes_per_class": shapes32,
                 "speedup_vs_f64_batched": el / el32,
                 "rel_l1_vs_f64": float(d32.sum() / u.abs().sum())}
    del b32, u32, d32

    # the plain path: one rktvd handle per problem, integrated one after the other
    plain_steps = max(1, min(args.steps, 5))
    odes = [hrweno.rktvd(p, p.ncells[0], 3) for p in probs]
    for o in odes:
        o.set_stream(stream.cuda_stream)
    views = [u[int(b.offsets[i]): int(b.offsets[i]) + int(b.ncells[i])] for i in range(BATCH_NPROB)]
    for i, o in enumerate(odes):  # warm-up: one step each
        o.integrate(views[i], 0.0, 0.5 * dts[i], dts[i])
    torch.cuda.synchronize()
    p0 = time.perf_counter()
    for i, o in enumerate(odes):
        o.integrate(views[i], 0.0, (plain_steps - 0.5) * dts[i], dts[i])
    torch.cuda.synchronize()
    plain = cells * plain_steps / (time.perf_counter() - p0)
    del odes, views

    # e2e: one batched step per call on pinned host memory
    uh = torch.from_numpy(packed.copy()).pin_memory()
    th = np.zeros(BATCH_NPROB)
    b.advance(uh, th, dts, 1)
    h0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 10))
    for _ in range(e2e_steps):
        b.advance(uh, th, dts, 1)
    e2e_el = dist.max(time.perf_counter() - h0)
    if dist.rank != 0:
        return None
    pk = peaks()
    achieved = BYTES_PER_CELL_UPDATE * cells * args.steps / el / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded multi-Gaussian u0 in [0, 1] per problem",
        "config": {"workload": f"batched_{BATCH_NPROB}_uneven_weno_lf_rk3", "problems": BATCH_NPROB,
                   "cells": cells, "sizes": "log-uniform [64, 65536]", "k": "2 or 3",
                   "numerics": "fast", "shapes_per_class": shapes,
                   "l2": f"inputs larger than L2: {cells * 24 >> 20} MiB of u, u1, u2"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": None, "peak_src": pk["src"]},
        "plain_per_problem": {"value": plain, "unit": UNIT, "steps": plain_steps,
                              "speedup_batched": value / plain},
        "forms": {"f32c": f32c_form},
        "cpu_baseline": None,
        "e2e": {"value": dist.world * cells * e2e_steps / e2e_el, "unit": UNIT,
                "h2d_bytes_per_step": 8 * b.size, "d2h_bytes_per_step": 8 * b.size},
        "gpu_launches": 3,
        "clocks": clk.summary(),
    }
    return line


# ------------------------------------------------------------------------------------------
# adjoint: gradient of J = 0.5 ||u(T) - u_target||^2 w.r.t. u0 on the 2^20-cell Burgers line,
# WENO5, fixed-alpha LF, RK3, 2000 steps, checkpoints every 45 steps; u_target from a forward
# run of a seeded perturbation of u0; one step here is one gradient evaluation
# ------------------------------------------------------------------------------------------
ADJ_N, ADJ_STEPS, ADJ_EVERY = 1 << 20, 2000, 45


def run_adjoint(args, dist: Dist) -> dict | None:
    import torch

    import hrweno
    from hrweno import workloads

    dev = dist.local if dist.world > 1 else 0
    torch.cuda.set_device(dev)
    n, nsteps = ADJ_N, args.adj_steps
    prob, u0h, dt = workloads.large_burgers(n, k=3)
    rng = np.random.default_rng(5)
    pert = 0.05 * workloads.multi_gaussian_1d(n, seed=9)
    stream = torch.cuda.Stream()
    adj = hrweno.adjoint(prob, checkpoint_every=ADJ_EVERY)
    adj.set_stream(stream.cuda_stream)
    u0 = torch.from_numpy(u0h).cuda()
    tgt = torch.empty_like(u0)
    adj.forward(u0 + torch.from_numpy(pert).cuda(), u0, dt, nsteps, uT=tgt)  # u_target
    J, g = adj.gradient(u0, tgt, dt, nsteps)  # warm-up
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    with ClockSampler(dev) as clk:
        e[0].record(stream)
        for _ in range(args.steps):
            J, g = adj.gradient(u0, tgt, dt, nsteps, grad=g)
        e[1].record(stream)
        e[2].record(stream)
        for _ in range(args.steps):
            adj.forward(u0, tgt, dt, nsteps)
        e[3].record(stream)
        torch.cuda.synchronize()
    t_grad = dist.max(e[0].elapsed_time(e[1]) * 1e-3 / args.steps)
    t_fwd = dist.max(e[2].elapsed_time(e[3]) * 1e-3 / args.steps)
    tape_bytes = adj.tape_bytes
    # central differences of the forward map in random directions
    fd = []
    fd_rough = []
    fd_norm = []  # |fd - g.d| / (|g| |d|): the error against the scale of the directional derivative
    xs = np.linspace(0.0, 1.0, n)
    for s in range(args.fd_directions):  # fourth-order central differences
        if s % 2 == 0:  # smooth random direction: 16 sine modes with random amplitudes, phases
            dh = np.zeros(n)
            for m in range(1, 17):
                dh += rng.standard_normal() * np.sin(np.pi * m * xs + rng.uniform(0, 2 * np.pi)) / m
        else:  # rough random direction: i.i.d. normal per cell
            dh = rng.standard_normal(n)
        d = torch.from_numpy(dh).cuda()
        h = 1e-5 * float(u0.abs().max()) / float(d.abs().max())
        Jv = [adj.forward(u0 + c * h * d, tgt, dt, nsteps)[0][0] for c in (2, 1, -1, -2)]
        fdv = (8.0 * (Jv[1] - Jv[2]) - (Jv[0] - Jv[3])) / (12.0 * h)
        gd = float((g * d).sum())
        (fd if s % 2 == 0 else fd_rough).append(abs(fdv - gd) / abs(gd))
        fd_norm.append(abs(fdv - gd) / (float(g.norm()) * float(d.norm())))
    # automatic segment length (checkpoint_every = 0)
    adj0 = hrweno.adjoint(prob, checkpoint_every=0)
    adj0.set_stream(stream.cuda_stream)
    J0, g0 = adj0.gradient(u0, tgt, dt, nsteps)
    torch.cuda.synchronize()
    e[0].record(stream)
    J0, g0 = adj0.gradient(u0, tgt, dt, nsteps, grad=g0)
    e[1].record(stream)
    torch.cuda.synchronize()
    t_tape = e[0].elapsed_time(e[1]) * 1e-3
    tape_every = adj0.checkpoint_every
    tape_bytes0 = adj0.tape_bytes
    same = bool(torch.equal(g0, g))
    gdiff = float((g0 - g).abs().max() / g.abs().max())
    del adj0, g0
    # a batch of 256 problems of 4096 cells, one gradient each, in one set of launches
    bn, bseg = 4096, 256
    bprob, _, bdt = workloads.large_burgers(bn, k=3, u0=np.ones(bn))
    bprob.alpha = (1.0, 1.0)
    bu0 = torch.from_numpy(np.concatenate(
        [workloads.multi_gaussian_1d(bn, seed=100 + s) / 2.0 for s in range(bseg)])).cuda()
    btg = bu0.flip(0).contiguous()
    badj = hrweno.adjoint(bprob, nseg=bseg, checkpoint_every=ADJ_EVERY)
    badj.set_stream(stream.cuda_stream)
    bJ, bg = badj.gradient(bu0, btg, bdt, nsteps)
    torch.cuda.synchronize()
    e[0].record(stream)
    bJ, bg = badj.gradient(bu0, btg, bdt, nsteps, grad=bg)
    e[1].record(stream)
    e[2].record(stream)
    badj.forward(bu0, btg, bdt, nsteps)
    e[3].record(stream)
    torch.cuda.synchronize()
    bt_grad, bt_fwd = e[0].elapsed_time(e[1]) * 1e-3, e[2].elapsed_time(e[3]) * 1e-3
    if dist.rank != 0:
        return None
    value = dist.world * n * nsteps / t_grad
    line = {
        "metric": METRIC, "value": value, "unit": UNIT + " (gradient)", "n_gpus": dist.world,
        "steps": args.steps, "warmup": 1, "ms_per_step": 1e3 * t_grad,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: 8-Gaussian u0, target = forward run of u0 + 0.05 x seeded Gaussians",
        "config": {"workload": f"adjoint_burgers1d_{n}_weno5_lf_rk3", "cells": n,
                   "time_steps": nsteps, "checkpoint_every": ADJ_EVERY, "alpha": "fixed max|u0|"},
        "adjoint": {"J": float(J[0]), "gradient_ms": 1e3 * t_grad, "forward_ms": 1e3 * t_fwd,
                    "cost_vs_forward": t_grad / t_fwd, "forward_steps_in_gradient": adj.forward_steps,
                    "segment_state_bytes": tape_bytes[0], "weno_tape_bytes": tape_bytes[1],
                    "auto_checkpointing": {"gradient_ms": 1e3 * t_tape, "cost_vs_forward": t_tape / t_fwd,
                                           "checkpoint_every": tape_every,
                                           "segment_state_bytes": tape_bytes0[0],
                                           "weno_tape_bytes": tape_bytes0[1],
                                           "same_gradient_bits": same,
                                           "max_rel_diff_vs_checkpointed": gdiff},
                    "fd_directions": args.fd_directions, "fd_order": 4,
                    "fd_max_rel_err_smooth": max(fd) if fd else None,
                    "fd_max_rel_err_rough": max(fd_rough) if fd_rough else None,
                    "fd_median_rel_err_rough": float(np.median(fd_rough)) if fd_rough else None,
                    "fd_max_err_over_norms": max(fd_norm) if fd_norm else None,
                    "batch": {"problems": bseg, "cells_each": bn, "gradient_ms": 1e3 * bt_grad,
                              "forward_ms": 1e3 * bt_fwd, "cost_vs_forward": bt_grad / bt_fwd,
                              "gradient_cell_updates_per_s": bseg * bn * nsteps / bt_grad}},
        "gpu_launches": None,
        "clocks": clk.summary(),
    }
    return line


# ------------------------------------------------------------------------------------------
# config1: the reference's own CPU-runnable case, 500 cells, driven like example1 (101 output
# times to t = 12, 1201 steps); one step is the whole driver loop
# ------------------------------------------------------------------------------------------
def run_config1(args, dist: Dist) -> dict | None:
    import torch

    import hrweno
    from hrweno import workloads

    dev = dist.local if dist.world > 1 else 0
    torch.cuda.set_device(dev)
    prob, u0 = workloads.burgers_config1()
    touts = [12.0 * ii / 100 for ii in range(101)]

    def loop(path: str, host: bool):
        """path "cluster": one cluster launch per integrate call (the default); "graphs": stage
        launches replayed from CUDA graphs; "stages": a launch per stage"""
        ode = hrweno.rktvd(prob, 500, 3)
        ode.set_cluster(path == "cluster")
        ode.set_graphs(path == "graphs")
        u = u0.copy() if host else torch.from_numpy(u0.copy()).cuda()
        t = 0.0
        t0 = time.perf_counter()
        for tout in touts:
            t = ode.integrate(u, t, tout, 1e-2)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, ode.nsteps

    for path in ("cluster", "graphs"):
        for _ in range(args.warmup):
            loop(path, False)
    res = {}
    for path in ("cluster", "graphs", "stages"):
        for host in (False, True):
            els = [loop(path, host)[0] for _ in range(args.steps)]
            res[(path, host)] = float(np.median(els))
    cells_steps = 500 * 1201
    cpu = None
    if not args.no_cpu:
        from oracle import oracle
        oracle.select_build("baseline")
        used = oracle.set_threads(1)
        o = oracle.ODE(prob, 500, 0, 3)
        u = u0.copy()
        t, c0 = 0.0, time.perf_counter()
        for tout in touts:
            t = o.integrate(u, t, tout, 1e-2)
        cel = time.perf_counter() - c0
        cpu = {"value": cells_steps / cel, "unit": UNIT, "cores": used, "kind": "port",
               "sample": f"the whole 1201-step driver loop ({cel * 1e3:.1f} ms), oracle, 1 thread"}
    if dist.rank != 0:
        return None
    line = {
        "metric": METRIC, "value": cells_steps / res[("cluster", False)], "unit": UNIT,
        "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * res[("cluster", False)], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "u0 = exp(-x^2) (the reference's example1)",
        "config": {"workload": "config1_burgers500_weno5_lf_rk3", "cells": 500, "time_steps": 1201,
                   "output_times": 101, "numerics": "fast"},
        "driver_loop_ms": {f"{'host' if host else 'device'}_{path}": 1e3 * v
                           for (path, host), v in res.items()},
        "cpu_baseline": cpu,
        "e2e": {"value": cells_steps / res[("cluster", True)], "unit": UNIT,
                "h2d_bytes_per_step": 8 * 500 * 101, "d2h_bytes_per_step": 8 * 500 * 101},
        "gpu_launches": 101,  # one cluster launch per integrate call
    }
    return line


def form_lines(name: str, d: dict) -> list:
    """Short JSON lines of a workload's result dict (its own line and its nested forms)."""
    out = []
    if name.startswith("pbe2d"):
        out.append({"form": f"{name}_fast", "value": d["value"], "ms": d["ms_per_step"],
                    "hbm_frac": d["roofline"]["frac"] if "roofline" in d else None})
        f = d["forms"].get("f32c")
        if f:
            out.append({"form": f"{name}_f32c", "value": f["value"], "ms": f["ms_per_step"],
                        "hbm_frac": f["hbm_frac"], "moved_B": f["moved_bytes_per_cell_update"],
                        "l1_vs_fast": f["rel_l1_vs_f64"]})
    elif name == "batched":
        out.append({"form": "batched_4096_fast", "value": d["value"], "ms": d["ms_per_step"],
                    "cells": d["config"]["cells"],
                    "x_plain_per_problem": d["plain_per_problem"]["speedup_batched"]})
        f = d["forms"]["f32c"]
        out.append({"form": "batched_4096_f32c", "value": f["value"], "ms": f["ms_per_step"],
                    "x_fast_batched": f["speedup_vs_f64_batched"], "l1_vs_fast": f["rel_l1_vs_f64"]})
    elif name == "adjoint":
        a = d["adjoint"]
        out.append({"form": "adjoint_2^20_2000steps", "grad_ms": a["gradient_ms"],
                    "fwd_ms": a["forward_ms"], "cost_vs_fwd": a["cost_vs_forward"],
                    "fd_dirs": a["fd_directions"], "fd_max_rel": max(a["fd_max_rel_err_smooth"] or 0,
                                                                     a["fd_max_rel_err_rough"] or 0),
                    "batch256x4096_cost_vs_fwd": a["batch"]["cost_vs_forward"]})
    elif name == "config1":
        ms = d["driver_loop_ms"]
        out.append({"form": "config1_500x1201", "ms_cluster": ms["device_cluster"],
                    "ms_stage_graphs": ms["device_graphs"], "ms_host_arrays": ms["host_cluster"],
                    "ms_cpu_1core": (500 * 1201 / d["cpu_baseline"]["value"] * 1e3
                                     if d.get("cpu_baseline") else None)})
    return out


def main() -> None:
    global NC
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 200 burgers1d, 100 pbe2d, 20 batched, 2 adjoint "
                         "gradients, 3 config1 runs)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--forms", default="line,k2,pbe2d,batched,adjoint,config1",
                    help="comma-separated forms printed before the headline line (line: the "
                         "plain FP64 and compensated FP32 forms of the same line; k2: the line "
                         "with WENO3; pbe2d: the 4096^2 and 1024^2 grids; the others: their "
                         "workloads)")
    ap.add_argument("--no-forms", action="store_true", help="same as --forms ''")
    ap.add_argument("--workload", default="burgers1d", choices=["burgers1d", "pbe2d", "batched", "adjoint", "config1"],
                    help="burgers1d (default): the 2^24-cell line; pbe2d: the 2D PBE grid")
    ap.add_argument("--pbe-n", type=int, default=PBE_N, help="pbe2d grid size per dimension")
    ap.add_argument("--adj-steps", type=int, default=ADJ_STEPS, help="adjoint: time steps")
    ap.add_argument("--fd-directions", type=int, default=64,
                    help="adjoint: random directions of the central-difference check (64 as the "
                         "adjoint configuration states; the default burgers1d run checks 2)")
    ap.add_argument("--cells", type=int, default=NC,
                    help="cells of the line (default 2^24, the benchmark workload; smaller "
                         "lines are for profiler captures)")
    args = ap.parse_args()
    args.forms = set() if args.no_forms else {f for f in args.forms.split(",") if f}
    if args.steps is None:
        args.steps = {"burgers1d": 200, "pbe2d": 100, "batched": 20, "adjoint": 2,
                      "config1": 3}[args.workload]
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    NC = args.cells
    if args.impl == "reference":
        # CPU arm: rank 0 alone runs; no process group is needed
        if int(os.environ.get("RANK", "0")) == 0:
            run_reference(args)
        return
    dist = Dist()
    try:
        runs = {"pbe2d": run_pbe2d, "batched": run_batched, "adjoint": run_adjoint,
                "config1": run_config1}
        if args.workload != "burgers1d":
            line = runs[args.workload](args, dist)
            if line is not None and dist.rank == 0:
                print(json.dumps(line), flush=True)
            return
        line, forms = run_ours(args, dist)
        # the other forms of the metric, each on its own workload, one short line each
        sub = argparse.Namespace(**vars(args))
        sub.steps, sub.no_cpu = min(args.steps, 100), True
        if "k2" in args.forms:
            forms += run_line_forms(sub, dist, 2)
        if "pbe2d" in args.forms:
            for n in (PBE_N, 1024):
                sp = argparse.Namespace(**vars(sub))
                sp.pbe_n = n
                pb = run_pbe2d(sp, dist)
                if pb is not None:
                    forms += form_lines(f"pbe2d_{n}", pb)
        if "batched" in args.forms:
            sb = argparse.Namespace(**vars(sub))
            sb.steps = min(args.steps, 20)
            bt = run_batched(sb, dist)
            if bt is not None:
                forms += form_lines("batched", bt)
        if "adjoint" in args.forms:
            sa = argparse.Namespace(**vars(sub))
            sa.steps, sa.fd_directions = 1, 2
            ad = run_adjoint(sa, dist)
            if ad is not None:
                forms += form_lines("adjoint", ad)
        if "config1" in args.forms:
            sc = argparse.Namespace(**vars(sub))
            sc.steps, sc.no_cpu = 3, args.no_cpu
            c1 = run_config1(sc, dist)
            if c1 is not None:
                forms += form_lines("config1", c1)
        if dist.rank == 0:
            for f in forms:
                print(json.dumps(f, separators=(",", ":")), flush=True)
            if line is not None:
                line["forms"] = [f["form"] for f in forms]
                print(json.dumps(line), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
