#!/usr/bin/env python3
"""Throughput benchmark of the wolfd2 projection-method time step on GB300.

Workload (one "step" = one pass of main.f:690-972, the whole time step):
lid-driven cavity, 1024 x 1024 uniform cells, Re = 1000, seeded divergence-
free perturbation (16 x 16 streamfunction modes, N(0, 1e-3) amplitudes),
red/black point SOR, plain FP64.  dt = 2.5e-4: at the named dt = 1e-3 the
reference's own Newton-Kantorovich iteration diverges to NaN in the first
step at this resolution (the mechanical translation of the reference source,
the CPU oracle and the GPU path all agree on that), and at 5e-4 it drifts
unstable within ten steps; dt = 2.5e-4 keeps the viscous number
dt/(h^2 Re) of the stable 512x512 case and runs the reference algorithm
cleanly (7-11 Q-L iterations and the full 2000 SOR sweeps per step).

Arms:
  --impl ours       the CUDA library through its C-ABI (value: device-timed
                    with CUDA events on the library stream; e2e: host buffers
                    with the H2D/D2H copies inside the timed region)
  --impl reference  the reference algorithm on the host cores (the CPU
                    oracle's restatement; no Fortran compiler exists on the
                    GPU machines to build the reference itself)

Multi-GPU: the single-case path does not shard (per-sweep halos, global
max-norms and domain-long chains), so N GPUs run N independent replicas and
`value` sums them ("replicas only", scaling weak).
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from wolfd2_gb300 import deck  # noqa: E402

METRIC = json.load(open(os.path.join(ROOT, "BASELINE.json")))["metric"]
UNIT = "cell-steps/s"
DT_NAMED = 1.0e-3


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples taken while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_case(args):
    return deck.cavity(args.n, args.re, args.dt, solver=args.solver)


def ppe_bytes(cells, nsor):
    """Algorithmic bytes of one Ppe call: RHS reads us, vs and writes b
    (3 words); each sweep reads p, b and writes p (3 words)."""
    return 8.0 * cells * (3 + 3 * nsor)


def mom_bytes(cells, nql):
    """Algorithmic bytes of one nAuxMomentum call: per Q-L iteration read us,
    vs, un, vn and write us, vs (6 words); chain systems stay on chip."""
    return 8.0 * cells * 6 * nql


def step_bytes(cells, nql, nsor):
    return 8.0 * cells * (6 * nql + 3 + 3 * nsor + 5 + 3)


def reference_runner(case, ic):
    """The host-side reference run: the mechanical translation of the
    reference's Fortran source (oracle/f77ref.py, kind "reference") when its
    generated C is present, else the oracle's restatement (kind "port").
    Both are the serial reference algorithm on one host core."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import f77ref
    import oracle as O
    u, v, p = ic
    fields = {"u": u, "v": v, "p": p}
    try:
        if f77ref.build(case.nx + 1, case.ny + 1):
            import refrun
            return refrun.RefRun(case, fields=fields, cold_start=False), "reference", \
                "mechanical F77->C translation of the reference source, gcc -O2, 1 thread"
    except Exception:  # no translation on this machine: fall back to the restatement
        pass
    return O.OracleRun(case, fields=fields, cold_start=False), "port", \
        "C restatement of the reference (oracle), gcc -O2, 1 thread"


def cpu_step_sample(case, ic, nsteps=1):
    """Time `nsteps` full reference steps on the host; returns
    (cell-steps/s, seconds, threads, kind, how)."""
    r, kind, how = reference_runner(case, ic)
    t0 = time.perf_counter()
    r.step(nsteps)
    dt = time.perf_counter() - t0
    return case.cells * nsteps / dt, dt, 1, kind, how


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    case = make_case(args)
    ic = deck.perturbation_ic(case, args.seed)
    r, kind, how = reference_runner(case, ic)
    r.step(args.warmup)
    t0 = time.perf_counter()
    r.step(args.steps)
    dt = time.perf_counter() - t0
    value = case.cells * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(args, case),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": kind,
                         "sample": f"{args.warmup} + {args.steps} full time steps of the same case; {how}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "iterations": [[h[0], h[1]] for h in r.history[-args.steps:]],
    }
    print(json.dumps(line), flush=True)


def config_of(args, case):
    return {"workload": (f"lid-driven cavity {args.n}x{args.n} cells, Re={args.re:g}, "
                         f"dt={args.dt:g} (the named dt={DT_NAMED:g} drives the reference scheme to NaN at this size), "
                         f"seeded 16x16-mode streamfunction perturbation (seed {args.seed}), "
                         f"ppe_solver {args.solver}, plain FP64"),
            "cells": case.cells, "nx": case.nx, "ny": case.ny, "re": args.re, "dt": args.dt,
            "ppe_solver": args.solver,
            "l2": "flushed between timed steps (256 MiB write); per-step working set > 2x L2"}


def run_ours(args):
    import torch
    import torch.distributed as dist
    from wolfd2_gb300.gpu import K_COPY, K_MOMENTUM, K_POST, K_PPE, K_BC, KERNEL_NAMES, Solver

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    case = make_case(args)
    u0, v0, p0 = deck.perturbation_ic(case, args.seed + rank)
    s = Solver.for_case(case)
    if args.threads or args.blocks_per_sm or args.seg or args.warm:
        s.tune(seg=args.seg, warm=args.warm, threads=args.threads, blocks_per_sm=args.blocks_per_sm)
    prm = case.params
    st = torch.cuda.ExternalStream(s.stream(), device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    # warm-up
    s.load_fields(u0, v0, p0)
    hist = s.step(prm, args.warmup) if args.warmup else []
    barrier()

    # device-timed region: fields resident in HBM
    s.profile(True)
    n_launch0 = s.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier()
        t_wall0 = time.perf_counter()
        for k in range(args.steps):
            with torch.cuda.stream(st):
                flush.fill_(float(k))
                ev[k][0].record(st)
            hist += s.step(prm, 1)
            with torch.cuda.stream(st):
                ev[k][1].record(st)
        barrier()
        t_wall = time.perf_counter() - t_wall0
    launches = s.launch_count() - n_launch0
    chain_rounds, chain_fallbacks = s.chain_stats()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_dev = sum(step_ms) / 1e3
    prof = {k: s.profile_read(k) for k in (K_MOMENTUM, K_PPE, K_POST, K_BC, K_COPY)}
    s.profile(False)
    timed = hist[-args.steps:]

    # end-to-end through the C-ABI with host buffers, copies in the timed region
    u, v, p = s.store_fields()
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.load_fields(u, v, p)
        s.step(prm, 1)
        u, v, p = s.store_fields()
    barrier()
    t_e2e = time.perf_counter() - t0
    field_bytes = (case.nx + 2) * (case.ny + 2) * 8

    # max over ranks
    t_max = t_dev
    t_e2e_max = t_e2e
    if world > 1:
        tt = torch.tensor([t_dev, t_e2e], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max, t_e2e_max = float(tt[0]), float(tt[1])

    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    cells = case.cells
    value = world * cells * args.steps / t_max
    e2e_value = world * cells * e2e_steps / t_e2e_max
    hbm_peak, peak_kind = peaks()
    # dominant kernel: larger share of device time
    dom = max((K_MOMENTUM, K_PPE), key=lambda k: prof[k][0])
    nql = [h[0] if h[0] > 0 else 20 for h in timed]
    nsor = [h[1] for h in timed]
    if dom == K_PPE:
        alg = sum(ppe_bytes(cells, n) for n in nsor)
    else:
        alg = sum(mom_bytes(cells, n) for n in nql)
    dom_ms, dom_n = prof[dom]
    achieved = alg / (dom_ms / 1e3) / 1e9
    # FP64 pipe view of the red/black sweep: 11 add/mul + 1 divide per point
    sweep_pts = sum(cells * n for n in nsor)
    fp64 = None
    if prof[K_PPE][0] > 0:
        ops = sweep_pts * (11 + 8.9)
        fp64 = {"kernel": "k_ppe", "op_per_point": "11 add/mul + 1 div (div = 8.9 FMA slots)",
                "achieved_gops": ops / (prof[K_PPE][0] / 1e3) / 1e9, "peak_gops": 628.0,
                "peak_kind": "measured DFMA probe on this pool's GB300 (2 DFMA/clk/SM)",
                "frac": ops / (prof[K_PPE][0] / 1e3) / 1e9 / 628.0}
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        tj = json.load(open(tpath)).get(KERNEL_NAMES[dom])
        if tj:
            # scale a captured small case by the units processed per launch
            traffic = tj["bytes_per_unit"] * (alg / dom_n) / tj["alg_bytes_per_unit"]
    cpu = None
    if not args.no_cpu_baseline:
        cv, csec, cores, kind, how = cpu_step_sample(case, (u0, v0, p0), 1)
        cpu = {"value": cv, "unit": UNIT, "cores": cores, "kind": kind,
               "sample": f"1 full time step of the same {args.n}x{args.n} case from the same initial state "
                         f"({csec:.1f} s); {how}"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_of(args, case),
        "parallelism": "replicas only" if world > 1 else "single GPU",
        "roofline": {"bound": "hbm", "kernel": KERNEL_NAMES[dom], "achieved": achieved,
                     "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                     "peak_kind": peak_kind, "traffic": traffic,
                     "alg_bytes_per_launch": alg / dom_n, "avg_launch_ms": dom_ms / dom_n},
        "fp64_roof": fp64,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 3 * field_bytes,
                "d2h_bytes_per_step": 3 * field_bytes, "steps": e2e_steps},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": launches,
        "kernel_ms": {KERNEL_NAMES[k]: {"total_ms": v[0], "launches": v[1]} for k, v in prof.items()},
        "iterations": [[h[0], h[1]] for h in timed],
        "chain": {"max_verify_rounds": chain_rounds, "sequential_fallbacks": chain_fallbacks,
                  "segment_rows": s.seg if hasattr(s, "seg") else None},
        "wall_s": t_wall,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=1024, help="cells per side")
    ap.add_argument("--re", type=float, default=1000.0)
    ap.add_argument("--dt", type=float, default=2.5e-4)
    ap.add_argument("--solver", default="rb_sor", choices=sorted(deck.PPE_SOLVERS))
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--threads", type=int, default=0, help="threads per block (0: library default)")
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--seg", type=int, default=0, help="chain segment rows (0: auto)")
    ap.add_argument("--warm", type=int, default=0, help="chain warm-up rows (0: default)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
