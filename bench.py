#!/usr/bin/env python3
"""Throughput benchmark of the wolfd2 projection-method time step on GB300.

Workload (one "step" = one pass of main.f:690-972, the whole time step):
lid-driven cavity, 1024 x 1024 uniform cells, Re = 1000, seeded divergence-
free perturbation (16 x 16 streamfunction modes, N(0, 1e-3) amplitudes),
red/black point SOR with the Poisson solve converged: sor_relaxation at the
model problem's optimum 2/(1 + sin(pi/1024)) (rounded to FP32, so both
precisions relax by the same factor), sor_tolerance 1e-9, max_sor_iter
20000 -- the reference's own keywords -- which brings the interior
divergence (dk times the Poisson residual) below 1e-10 in both precisions.
dt = 2.5e-4: at the named dt = 1e-3 the reference's own Newton-Kantorovich
iteration diverges to NaN in the first step at this resolution (the
mechanical translation of the reference source, the CPU oracle and the GPU
path all agree on that), and at 5e-4 it drifts unstable within ten steps;
dt = 2.5e-4 keeps the viscous number dt/(h^2 Re) of the stable 512x512 case.
--ppe-defaults runs the reference's default Poisson settings instead
(sorrel 1, sortol 1e-8, 2000 sweeps: unconverged at this size).

Arms:
  --impl ours       the CUDA library through its C-ABI (value: device-timed
                    with CUDA events on the library stream; e2e: host buffers
                    with the H2D/D2H copies inside the timed region)
  --impl reference  the reference algorithm on one host core: the
                    mechanical translation of the reference's Fortran source
                    to C (no Fortran compiler exists on the GPU machines),
                    full time steps of the same case, as many as fit a
                    bounded time

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

METRIC = "cell-steps/s, mixed FP32+refine vs plain FP64 on GB300 at <=1e-10 div; % HBM roof"
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


# Plane channel of the benchmark: 4096 x 1024 cells, length 4 x height 1,
# Re = 5000 on the half-height (10000 on the height, the deck's length
# scale), dt = 2.5e-4, parabolic + seeded Fourier inflow (amplitude 1e-2).
CHANNEL = {"ncx": 4096, "ncy": 1024, "re": 10000.0, "dt": 2.5e-4}


THERMAL = {"nmeiter": 2, "dmeittol": 0.0, "pr": 0.71, "fr": 0.05}


def optimal_relaxation(n):
    """SOR's optimal relaxation for the n x n model Poisson problem,
    2/(1 + sin(pi/n)), rounded to the nearest FP32 value so that the FP64
    and FP32 sweeps relax by the same factor."""
    return float(np.float32(2.0 / (1.0 + np.sin(np.pi / n))))


def poisson_settings(args):
    """(sorrel, sortol, msorit) of the run: converged by default for the
    cavity workload, the reference's defaults (parse.f:136,160-161) with
    --ppe-defaults or for the other workloads."""
    if args.workload == "cavity" and not args.ppe_defaults:
        sorrel = args.sorrel or optimal_relaxation(args.n)
        return sorrel, args.sortol or 1.0e-9, args.msorit or 20000
    return args.sorrel or 1.0, args.sortol or 1.0e-8, args.msorit or 2000


def make_case(args):
    if args.workload == "channel":
        case = deck.channel_inflow(CHANNEL["ncx"], CHANNEL["ncy"], CHANNEL["re"], CHANNEL["dt"],
                                   seed=args.seed, solver=args.solver)
    elif args.workload == "clustered":
        case = deck.clustered_cavity(args.n, args.re, args.dt, solver=args.solver)
    elif args.workload == "thermal":
        case = deck.heated_cavity(args.n, args.re, args.dt, solver=args.solver, pr=THERMAL["pr"],
                                  fr=THERMAL["fr"], nmeiter=THERMAL["nmeiter"], dmeittol=THERMAL["dmeittol"])
    else:
        case = deck.cavity(args.n, args.re, args.dt, solver=args.solver)
    case.params.sorrel, case.params.sortol, case.params.msorit = poisson_settings(args)
    return case


def make_ic(args, case, rank=0):
    if args.workload == "channel":
        return deck.channel_ic(case)
    return deck.perturbation_ic(case, args.seed + rank)


def make_t0(case):
    """Initial temperature of the heated cavity: linear from the hot west
    wall (1) to the cold east wall (0) over the cell centres."""
    t = np.zeros((case.nx + 2, case.ny + 2), order="F")
    t[...] = (1.0 - (np.arange(case.nx + 2) - 0.5) / (case.nx - 1))[:, None]
    return np.asfortranarray(np.clip(t, 0.0, 1.0))


def ppe_bytes(cells, nsor):
    """Algorithmic bytes of one Ppe call: RHS reads us, vs and writes b
    (3 words); each sweep reads p, b and writes p (3 words)."""
    return 8.0 * cells * (3 + 3 * nsor)


def mom_bytes(cells, nql, word=8):
    """Algorithmic bytes of one nAuxMomentum call: per Q-L iteration read us,
    vs, un, vn and write us, vs (6 words of `word` bytes: 8 plain, 4 in the
    mixed path's FP32 momentum); chain systems stay on chip."""
    return float(word) * cells * 6 * nql


def step_bytes(cells, nql, nsor):
    return 8.0 * cells * (6 * nql + 3 + 3 * nsor + 5 + 3)


def reference_runner(case, ic, t0=None):
    """The host-side reference run: the mechanical translation of the
    reference's Fortran source (oracle/f77ref.py, kind "reference") when its
    generated C is present, else the oracle's restatement (kind "port").
    Both are the serial reference algorithm on one host core."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import f77ref
    import oracle as O
    u, v, p = ic
    fields = {"u": u, "v": v, "p": p}
    if t0 is not None:
        fields["t"] = t0
    if getattr(case.regions, "profiles", None):
        # the reference has no per-row inflow: time the restatement with the shim
        return O.OracleRun(case, fields=fields, cold_start=False), "port", \
            "C restatement of the reference (oracle) with the inflow-profile shim, gcc -O2, 1 thread"
    try:
        if f77ref.build(case.nx + 1, case.ny + 1):
            import refrun
            return refrun.RefRun(case, fields=fields, cold_start=False), "reference", \
                "mechanical F77->C translation of the reference source, gcc -O2, 1 thread"
    except Exception:  # no translation on this machine: fall back to the restatement
        pass
    return O.OracleRun(case, fields=fields, cold_start=False), "port", \
        "C restatement of the reference (oracle), gcc -O2, 1 thread"


def cpu_step_sample(case, ic, nsteps=1, t0=None, with_run=False):
    """Time `nsteps` full reference steps on the host; returns
    (cell-steps/s, seconds, threads, kind, how) and, with_run, the run
    itself (its fields and per-step counts)."""
    r, kind, how = reference_runner(case, ic, t0)
    t0 = time.perf_counter()
    r.step(nsteps)
    dt = time.perf_counter() - t0
    out = (case.cells * nsteps / dt, dt, 1, kind, how)
    return out + (r,) if with_run else out


def run_reference_sampled(args):
    """Reference arm of the ensemble and adjoint workloads: the reference's
    forward steps on one host core over a bounded sample of the workload
    (the reference has neither batching nor an adjoint)."""
    if args.workload == "ensemble":
        members = ensemble_members(args)
        cases = [(m.case, deck.perturbation_ic(m.case, args.seed + i)) for i, m in enumerate(members)]
        config = ensemble_config(args, members, args.refine_sweeps or 64, not args.no_graph)
    else:
        case = deck.cavity(ADJOINT["n"], ADJOINT["re"], ADJOINT["dt"], solver="rb_sor")
        cases = [(case, deck.perturbation_ic(case, args.seed))]
        config = {"workload": f"adjoint workload's forward: lid-driven cavity {ADJOINT['n']}x{ADJOINT['n']}, "
                              f"Re={ADJOINT['re']:g}, dt={ADJOINT['dt']:g}, rb_sor, plain FP64"}
    done, secs, steps_run, kind, how = 0, 0.0, 0, "port", ""
    for step_round in range(max(1, args.steps)):
        for c, ic in cases:
            r, kind, how = reference_runner(c, ic)
            t0 = time.perf_counter()
            r.step(1)
            secs += time.perf_counter() - t0
            done += c.cells
            steps_run += 1
            if secs > 15.0 * max(1, args.steps):
                break
        if secs > 15.0 * max(1, args.steps):
            break
    value = done / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * secs / max(1, steps_run), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": kind,
                         "sample": f"{steps_run} single reference steps over the workload's cases in order "
                                   f"({done} cell-steps, {secs:.1f} s); {how}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload in ("ensemble", "adjoint"):
        run_reference_sampled(args)
        return
    case = make_case(args)
    ic = make_ic(args, case)
    r, kind, how = reference_runner(case, ic, make_t0(case) if args.workload == "thermal" else None)
    # a bounded sample: whole time steps from the initial state until the
    # step budget (--steps) or the time budget is used up; the host run
    # needs no warm-up
    budget = args.ref_seconds
    t0 = time.perf_counter()
    steps = 0
    while steps < max(1, args.steps):
        r.step(1)
        steps += 1
        if time.perf_counter() - t0 > budget:
            break
    dt = time.perf_counter() - t0
    value = case.cells * steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": steps, "warmup": 0,
        "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(args, case, args.refine_sweeps or 128),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": kind,
                         "sample": f"the first {steps} full time steps of the same case from the same "
                                   f"initial state ({dt:.1f} s, a budget of {budget:g} s or --steps "
                                   f"{args.steps}); {how}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "iterations": [[h[0], h[1]] for h in r.history[-steps:]],
    }
    print(json.dumps(line), flush=True)


def config_of(args, case, inner=None):
    prec = ("mixed: FP32 momentum (stencils, ADI chains) and FP32 red/black Poisson sweeps, "
            f"FP64 Poisson residual and correction ({inner} sweeps per refinement pass), FP64 "
            "divergence check, projection and norms; plain FP64 timed beside it"
            if args.precision == "mixed" else "plain FP64")
    if args.workload == "thermal":
        work = (f"differentially heated cavity {args.n}x{args.n} cells, Re={args.re:g}, dt={args.dt:g}, "
                f"energy equation on (Pe = Re x {THERMAL['pr']}), west wall t=1, east wall t=0, adiabatic "
                f"south/north, ideal-gas EqState density (tref 300, tmax 330) driving the buoyancy term at "
                f"Fr={THERMAL['fr']}, {THERMAL['nmeiter']} momentum/energy iterations per step "
                f"(dmeittol {THERMAL['dmeittol']:g}: all run), seeded 16x16-mode velocity perturbation "
                f"(seed {args.seed}), linear initial temperature, ppe_solver {args.solver}, plain FP64")
        re, dt = args.re, args.dt
    elif args.workload == "channel":
        work = (f"plane channel {CHANNEL['ncx']}x{CHANNEL['ncy']} cells, length 4 x height 1, "
                f"Re=5000 on the half-height (deck Re={CHANNEL['re']:g}), dt={CHANNEL['dt']:g}, "
                f"parabolic inflow + seeded 16-mode Fourier perturbation (amplitude 1e-2, seed {args.seed}) "
                f"as a per-row inlet profile, zero-gradient mass-conserving outlet (bound_cond.f BM_OUTLT2), "
                f"no-slip walls, ppe_solver {args.solver}, {prec}")
        re, dt = CHANNEL["re"], CHANNEL["dt"]
    elif args.workload == "clustered":
        work = (f"lid-driven cavity {args.n}x{args.n} cells clustered towards the walls (nodes s - 0.5 "
                f"sin(2 pi s)/(2 pi): cell widths 0.5/n to 1.5/n, no Poisson row the unit stencil), "
                f"Re={args.re:g}, dt={args.dt:g} (2.5e-4 drives the reference scheme to NaN on these cells), "
                f"seeded 16x16-mode streamfunction perturbation "
                f"(seed {args.seed}), ppe_solver {args.solver}, the reference's default Poisson settings, "
                f"{prec}; the mixed Poisson solve runs the general-row kernel")
        re, dt = args.re, args.dt
    else:
        prm = case.params
        conv = ("" if args.ppe_defaults else
                f" (the Poisson solve converged: interior divergence <= 1e-10 in both precisions)")
        work = (f"lid-driven cavity {args.n}x{args.n} cells, Re={args.re:g}, "
                f"dt={args.dt:g} (the named dt={DT_NAMED:g} drives the reference scheme to NaN at this size), "
                f"seeded 16x16-mode streamfunction perturbation (seed {args.seed}), "
                f"ppe_solver {args.solver}, sor_relaxation {prm.sorrel!r}, sor_tolerance {prm.sortol:g}, "
                f"max_sor_iter {prm.msorit}{conv}, {prec}")
        re, dt = args.re, args.dt
    prm = case.params
    return {"workload": work, "cells": case.cells, "nx": case.nx, "ny": case.ny, "re": re, "dt": dt,
            "ppe_solver": args.solver, "sor_relaxation": prm.sorrel, "sor_tolerance": prm.sortol,
            "max_sor_iter": prm.msorit, "precision": args.precision,
            "l2": "flushed between timed steps (256 MiB write); per-step working set > 2x L2"}


def ppe_bytes_general(cells, nsor):
    """Algorithmic bytes of one plain Ppe call with general rows: RHS reads
    us, vs and writes b (3 words); each sweep reads p, b, a1..a5 and writes p
    (8 words)."""
    return 8.0 * cells * (3 + 8 * nsor)


def mixed_ppe_bytes_general(cells, nsor, inner):
    """Algorithmic bytes of one mixed Ppe call with general rows: RHS reads
    us, vs and writes div (FP64, 24 B/cell); per refinement pass the residual
    reads p, div, a1..a5 (FP64) and writes r, e (FP32) = 64 B, the correction
    reads p, e and writes p = 20 B; each FP32 sweep reads e, r, c1..c5 and
    writes e = 32 B."""
    passes = -(-nsor // inner)
    return cells * (24.0 + passes * 84.0 + 32.0 * nsor)


def mixed_ppe_bytes(cells, nsor, inner):
    """Algorithmic bytes of one mixed Ppe call: RHS reads us, vs and writes b
    (FP64, 24 B/cell); per refinement pass the residual reads p, b (FP64) and
    writes r (FP32) = 20 B, each FP32 sweep reads e, r and writes e = 12 B,
    the correction reads p, e and writes p = 20 B."""
    passes = -(-nsor // inner)
    return cells * (24.0 + passes * 40.0 + 12.0 * nsor)


def run_arm(s, prm, args, precision, u0, v0, p0, st, flush, barrier, local, timed=True, t0=None):
    """Warm-up then `steps` device-timed steps of one precision mode from the
    same initial fields (and temperature t0 with the energy equation);
    returns the measurements and the final fields."""
    from wolfd2_gb300.gpu import K_BC, K_COPY, K_MOMENTUM, K_POST, K_PPE, K_THERM
    import torch
    kw = {"precision": precision, "refine_sweeps": args.refine_sweeps}
    s.load_fields(u0, v0, p0)
    if t0 is not None:
        s.load_thermal(t0)
    # single-step warm-up calls: the step's CUDA graphs (one per time-level
    # parity) are captured here, outside the timed region
    hist = []
    for _ in range(args.warmup):
        hist += s.step(prm, 1, **kw)
    barrier()
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
            hist += s.step(prm, 1, **kw)
            with torch.cuda.stream(st):
                ev[k][1].record(st)
        barrier()
        t_wall = time.perf_counter() - t_wall0
    launches = s.launch_count() - n_launch0
    t_dev = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    # per-kernel split: as many steps again, launched directly with events
    s.profile(True)
    for _ in range(args.steps):
        hist += s.step(prm, 1, **kw)
    kinds = (K_MOMENTUM, K_PPE, K_POST, K_BC, K_COPY) + ((K_THERM,) if t0 is not None else ())
    prof = {k: s.profile_read(k) for k in kinds}
    s.profile(False)
    fields = s.store_fields()
    if t0 is not None:
        fields = tuple(fields) + (s.store_thermal()[0],)
    # end-to-end through the C-ABI with pinned host buffers, the copies in
    # the timed region: each step loads u, v, p, runs, and reads them back
    pinned = [torch.empty((s.mny + 1, s.mnx + 1), dtype=torch.float64, pin_memory=True)
              for _ in range(len(fields))]
    host = [t.numpy().T for t in pinned]  # Fortran-ordered views of pinned memory
    for h, f in zip(host, fields):
        h[...] = f
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    barrier()
    tw0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.load_fields(*host[:3])
        if t0 is not None:
            s.load_thermal(host[3])
        s.step(prm, 1, **kw)
        s.store_fields(out=host[:3])
        if t0 is not None:
            s.store_thermal(out=host[3])
    barrier()
    t_e2e = time.perf_counter() - tw0
    return {"t_dev": t_dev, "t_e2e": t_e2e, "e2e_steps": e2e_steps, "hist": hist,
            "timed": hist[args.warmup:args.warmup + args.steps], "profiled": hist[-args.steps:],
            "prof": prof, "launches": launches,
            "clk": clk, "wall": t_wall, "fields": fields}


def kernel_name(kind, precision, tiled, thermal=False, general=False):
    """The kernel a profile kind stands for in this workload (general: the
    Poisson rows are not the unit stencil)."""
    from wolfd2_gb300.gpu import K_COPY, K_MOMENTUM, K_POST, K_PPE, K_THERM, KERNEL_NAMES
    if thermal and kind == K_POST:
        return "k_me_post+k_step_tail_th"
    if thermal and kind == K_COPY:
        return "k_copy_th"
    if kind == K_THERM:
        return "k_therm+k_eq_state"
    if kind == K_PPE:
        if precision == "mixed":
            # general rows on a Cartesian grid: the tiled general-row form
            return "k_ppe_mixgt" if general else "k_ppe_mixed"
        return "k_ppe_tiled" if tiled else "k_ppe"
    if kind == K_MOMENTUM:
        return "k_naux32" if precision == "mixed" else "k_naux"
    if kind == K_COPY and precision == "mixed":
        return "k_copy_mixed"
    return KERNEL_NAMES[kind]


FP64_PEAK_GOPS = 628.0


def roofline_of(arm, cells, precision, inner, tiled=True, sorrel=1.0, general=False):
    """Roofline of the dominant kernel of one arm (HBM view) and the FP64
    pipe view of the plain red/black sweep."""
    from wolfd2_gb300.gpu import K_MOMENTUM, K_PPE
    # the per-kernel times come from the profiled steps: their iteration counts
    prof, timed = arm["prof"], arm["profiled"]
    hbm_peak, peak_kind = peaks()
    dom = max((K_MOMENTUM, K_PPE), key=lambda k: prof[k][0])
    nql = [h[0] if h[0] > 0 else 20 for h in timed]
    nsor = [h[1] for h in timed]
    if dom == K_PPE:
        if precision == "mixed":
            mb = mixed_ppe_bytes_general if general else mixed_ppe_bytes
            alg = sum(mb(cells, n, inner) for n in nsor)
        else:
            alg = sum((ppe_bytes_general if general else ppe_bytes)(cells, n) for n in nsor)
    else:
        alg = sum(mom_bytes(cells, n, 4 if precision == "mixed" else 8) for n in nql)
    dom_ms, dom_n = prof[dom]
    # with momentum/energy iterations a step launches the kernel once per
    # iteration; the step record holds the last iteration's counts
    alg *= dom_n / max(1, len(timed))
    name = kernel_name(dom, precision, tiled, general=general)
    achieved = alg / (dom_ms / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        tj = json.load(open(tpath)).get(name)
        if tj:
            # a captured smaller case, scaled by the algorithmic bytes per launch
            traffic = tj["bytes_per_alg_byte"] * (alg / dom_n)
    roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak, "peak_kind": peak_kind, "traffic": traffic,
            "alg_bytes_per_launch": alg / dom_n, "avg_launch_ms": dom_ms / dom_n}
    fp64 = None
    if precision == "fp64" and prof[K_PPE][0] > 0 and not general:
        # unit-stencil red/black point: 4 subtractions, 1 multiply by -1/4,
        # 1 subtraction, the product by sorrel (when it is not 1) and 1
        # addition per point and sweep; the sweeps are the FP64 pipe's work
        relax = sorrel != 1.0
        per_point = 8.0 if relax else 7.0
        ops = sum(cells * n for n in nsor) * per_point
        gops = ops / (prof[K_PPE][0] / 1e3) / 1e9
        fp64 = {"bound": "fp64", "kernel": kernel_name(K_PPE, precision, tiled),
                "op_per_point": f"{per_point:g} FP64 add/mul (unit stencil{', relaxed' if relax else ''})",
                "achieved_gops": gops, "peak_gops": FP64_PEAK_GOPS,
                "peak_kind": "measured: FP64 fused multiply-add issue rate of the GB300 (2 per clock per SM "
                             "at 2070 MHz on 152 SMs), a probe run on the same hardware",
                "frac": gops / FP64_PEAK_GOPS,
                "roof_note": "the plain sweep's FP64 work per point takes longer than its 24 bytes of "
                             "traffic at the HBM rate, and its working set stays in L2: min(HBM, FP64) "
                             "is this roof"}
    return roof, fp64


def rel_max(a, b):
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def run_ours(args):
    import torch
    import torch.distributed as dist
    from wolfd2_gb300.gpu import PREC_FP64, PREC_MIXED, Solver

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    case = make_case(args)
    u0, v0, p0 = make_ic(args, case, rank)
    t0 = None
    if args.workload == "thermal":
        args.precision = "fp64"  # the loop with the energy equation is plain FP64
        t0 = make_t0(case)
    s = Solver.for_case(case)
    if args.no_tma:
        s.set_tma(False)
    if args.threads or args.blocks_per_sm or args.seg or args.warm:
        s.tune(seg=args.seg, warm=args.warm, threads=args.threads, blocks_per_sm=args.blocks_per_sm)
    if args.mixed_k or args.mixed_threads or args.mixed_mode:
        s.tune_mixed(args.mixed_k, args.mixed_threads, args.mixed_mode)
    inner = args.refine_sweeps or s.refine_sweeps or 16 * (args.mixed_k or 8)
    args.refine_sweeps = inner
    prm = case.params
    st = torch.cuda.ExternalStream(s.stream(), device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    arms = {}
    order = ["fp64", "mixed"] if args.precision == "mixed" else ["fp64"]
    for name in order:
        arms[name] = run_arm(s, prm, args, PREC_MIXED if name == "mixed" else PREC_FP64,
                             u0, v0, p0, st, flush, barrier, local, t0=t0)
    head = arms[args.precision]

    # max over ranks
    t_max, t_e2e_max = head["t_dev"], head["t_e2e"]
    if world > 1:
        tt = torch.tensor([t_max, t_e2e_max], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max, t_e2e_max = float(tt[0]), float(tt[1])

    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    cells = case.cells
    field_bytes = (case.nx + 2) * (case.ny + 2) * 8
    nfields = 4 if t0 is not None else 3
    value = world * cells * args.steps / t_max
    e2e_value = world * cells * head["e2e_steps"] / t_e2e_max
    # the plain path's red/black solve runs on shared-memory tiles at this size
    tiled = args.solver in ("rb_sor", "par_rb_sor") and cells >= 152 * 1024 and args.workload != "clustered"
    general = args.workload == "clustered"
    roof, fp64 = roofline_of(head, cells, args.precision, inner, tiled, prm.sorrel, general)
    plain = None
    accuracy = None
    if args.precision == "mixed":
        a64 = arms["fp64"]
        r64, f64 = roofline_of(a64, cells, "fp64", inner, tiled, prm.sorrel, general)
        plain = {"value": world * cells * args.steps / a64["t_dev"], "unit": UNIT,
                 "ms_per_step": 1e3 * a64["t_dev"] / args.steps,
                 "e2e": world * cells * a64["e2e_steps"] / a64["t_e2e"],
                 "roofline": r64, "fp64_roof": f64, "gpu_launches": a64["launches"],
                 "kernel_ms": {kernel_name(k, "fp64", tiled, general=general): {"total_ms": v[0], "launches": v[1]}
                               for k, v in a64["prof"].items()},
                 "iterations": [[h[0], h[1]] for h in a64["timed"]],
                 "clocks": a64["clk"].summary()}
        fm, fp = head["fields"], a64["fields"]
        errs = {nm: rel_max(a, b) for nm, a, b in zip("uvp", fm, fp)}
        vscale = max(float(np.max(np.abs(fp[0]))), float(np.max(np.abs(fp[1]))), 1e-300)
        vel_rel = max(float(np.max(np.abs(fm[0] - fp[0]))), float(np.max(np.abs(fm[1] - fp[1])))) / vscale
        # pressure on the dynamic-pressure scale (velocity scale squared), or max |p| when larger
        pscale = max(float(np.max(np.abs(fp[2]))), vscale * vscale)
        p_dyn = float(np.max(np.abs(fm[2] - fp[2]))) / pscale
        div_m = [h[3] for h in head["hist"]]
        div_p = [h[3] for h in a64["hist"]]
        divi_m = max(h[4] for h in head["hist"])
        divi_p = max(h[4] for h in a64["hist"])
        accuracy = {
            "against": "plain FP64 path after the same warm-up + timed steps from the same initial "
                       "state (bit-identical to the FP64 oracle: parity tests)",
            "steps": len(head["hist"]),
            "velocity_rel_maxnorm": vel_rel,
            "u_rel_maxnorm": errs["u"], "v_rel_maxnorm": errs["v"], "p_rel_maxnorm": errs["p"],
            "p_rel_dynamic": p_dyn,
            "divmax_interior_mixed": divi_m, "divmax_interior_fp64": divi_p,
            "divmax_mixed": max(div_m), "divmax_fp64": max(div_p),
            "divmax_rel_diff": abs(max(div_m) - max(div_p)) / max(max(div_p), 1e-300),
            "divergence_note": "interior: cells whose four neighbours are Poisson unknowns and whose "
                               "faces Project sets, where the divergence is dk times the Poisson "
                               "residual; divmax: all pressure cells, which adds at the boundary "
                               "dk * coefficient * (change of the ghost pressure Ppe holds frozen "
                               "during the solve) -- the reference scheme's, in both precisions",
            "velocity_within_1e-5": vel_rel <= 1e-5,
            "div_le_1e-10": divi_m <= 1e-10 and divi_p <= 1e-10,
        }
    cpu = None
    parity = None
    if not args.no_cpu_baseline:
        cv, csec, cores, kind, how, ref = cpu_step_sample(case, (u0, v0, p0), 1, t0, with_run=True)
        cpu = {"value": cv, "unit": UNIT, "cores": cores, "kind": kind,
               "sample": f"1 full time step of the same {case.nx - 1}x{case.ny - 1} case from the same initial "
                         f"state ({csec:.1f} s); {how}"}
        if t0 is None:
            # the same first step on the GPU's plain FP64 path, field for field
            s.load_fields(u0, v0, p0)
            h1 = s.step(prm, 1, precision=PREC_FP64)
            g = s.store_fields()
            parity = {"against": f"{how.split(',')[0]} ({kind}): 1 time step of this case from the same "
                                 "initial state, plain FP64 path",
                      "iterations_equal": [h1[0][0], h1[0][1]] == list(ref.history[0][:2]),
                      "iterations": [h1[0][0], h1[0][1]]}
            for nm, a in zip("uvp", g):
                parity[nm] = rel_max(a, ref.f[nm])
            parity["bitwise"] = all(np.array_equal(a, ref.f[nm]) for nm, a in zip("uvp", g))
    chain_rounds, chain_fallbacks = s.chain_stats()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
        "steps_per_s": world * args.steps / t_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64",
        "data": "synthetic", "config": config_of(args, case, inner),
        "parallelism": "replicas only" if world > 1 else "single GPU",
        "roofline": roof,
        "fp64_roof": fp64,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nfields * field_bytes,
                "d2h_bytes_per_step": nfields * field_bytes, "steps": head["e2e_steps"],
                "host_buffers": "pinned"},
        "plain_fp64": plain,
        "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
        "accuracy": accuracy,
        "parity": parity,
        "cpu_baseline": cpu,
        "clocks": head["clk"].summary(),
        "gpu_launches": head["launches"],
        "kernel_ms": {kernel_name(k, args.precision, tiled, t0 is not None, general): {"total_ms": v[0],
                                                                                      "launches": v[1]}
                      for k, v in head["prof"].items()},
        "iterations": [[h[0], h[1]] for h in head["timed"]],
        "chain": {"max_verify_rounds": chain_rounds, "sequential_fallbacks": chain_fallbacks},
        "wall_s": head["wall"],
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


ADJOINT = {"n": 256, "re": 400.0, "dt": 2.0e-3, "steps": 400, "every": 20, "eps": 1.0e-6}


def run_adjoint(args):
    """The adjoint workload: gradient of J = 0.5 h^2 sum(u^2 + v^2) at the final step
    with respect to the initial u, v and the 256-point lid profile, by the
    library's discrete adjoint (checkpoint and recompute), checked against
    central finite differences of the same map along seeded directions."""
    import torch
    from wolfd2_gb300.gpu import Solver

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    NORTH, WEST, VAR_U = 4, 1, 1
    if args.adj_case == "channel":
        # the channel's gradient: final kinetic energy w.r.t. the inflow profile;
        # the start is the flow after two steps (v = 0 everywhere at the
        # initial field puts every v-driven upwind selector on its branch point)
        case = deck.channel_inflow(CHANNEL["ncx"], CHANNEL["ncy"], CHANNEL["re"], CHANNEL["dt"], seed=args.seed)
        n = CHANNEL["ncy"]
        nsteps = args.adj_steps if args.adj_steps != ADJOINT["steps"] else 10
        every = 5
        face = (1, 1, WEST, VAR_U)
        lid = case.regions.profiles[(1, 1, WEST, VAR_U)].copy()
        s0 = Solver.for_case(case, tuned=False)
        s0.load_fields(*deck.channel_ic(case))
        s0.step(case.params, 2)
        u0, v0, p0 = s0.store_fields()
        s0.close()
    else:
        n, nsteps, every = ADJOINT["n"], args.adj_steps, ADJOINT["every"]
        case = deck.cavity(n, ADJOINT["re"], ADJOINT["dt"], solver="rb_sor")
        u0, v0, p0 = deck.perturbation_ic(case, args.seed)
        lid = np.ones(case.nx + 2)
        face = (1, 1, NORTH, VAR_U)
    prm = case.params
    w = (1.0 / n) ** 2

    def solver():
        s = Solver.for_case(case, tuned=False)
        s.set_face_profile(*face, lid)
        return s

    s = solver()
    s.load_fields(u0, v0, p0)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        J, gu, gv, gp, gl, counts = s.adjoint(prm, nsteps, every, w, profile=face, nprof=lid.size)
        t_adj = time.perf_counter() - t0
    launches = s.launch_count()
    # forward alone, the same steps (frozen counts), for the adjoint's cost ratio
    s.load_fields(u0, v0, p0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.step_counts(prm, counts)
    t_fwd = time.perf_counter() - t0

    def objective(u, v):
        nx, ny = case.nx, case.ny
        return 0.5 * w * (np.sum(u[1:nx + 1, 2:ny + 1] ** 2) + np.sum(v[2:nx + 1, 1:ny + 1] ** 2))

    def J_at(u, v, lidv):
        s.set_face_profile(*face, lidv)
        s.load_fields(np.asfortranarray(u), np.asfortranarray(v), p0)
        s.step_counts(prm, counts)
        uu, vv, _ = s.store_fields()
        return objective(uu, vv)

    # seeded directions in the interior unknowns of u0, v0 and in the lid
    rng = np.random.default_rng(args.seed + 1)
    nx, ny = case.nx, case.ny
    mu = np.zeros_like(u0, dtype=bool)
    mv = np.zeros_like(mu)
    mu[2:nx, 2:ny + 1] = True
    mv[2:nx + 1, 2:ny] = True
    eps = ADJOINT["eps"]
    extra_eps = [float(x) for x in args.fd_eps.split(",") if x] if args.fd_eps else []
    errs, errs4, pairs, sweep = [], [], [], {}
    t0 = time.perf_counter()
    for _ in range(args.fd_dirs):
        du = np.where(mu, rng.normal(size=u0.shape), 0.0)
        dv = np.where(mv, rng.normal(size=v0.shape), 0.0)
        dl = rng.normal(size=lid.shape)
        if args.adj_case == "channel":
            dl[:2] = 0.0          # rows outside the channel carry no inflow
            dl[case.ny + 1:] = 0.0
        ad = float(np.sum(gu * du) + np.sum(gv * dv) + np.sum(gl * dl))
        for e_ in [eps] + extra_eps:
            Jp = J_at(u0 + e_ * du, v0 + e_ * dv, lid + e_ * dl)
            Jm = J_at(u0 - e_ * du, v0 - e_ * dv, lid - e_ * dl)
            fd = (Jp - Jm) / (2 * e_)
            fd4 = None
            if args.fd_order == 4:
                # fourth-order central difference: cancels the eps^2
                # truncation term of the two-point one
                J2p = J_at(u0 + 2 * e_ * du, v0 + 2 * e_ * dv, lid + 2 * e_ * dl)
                J2m = J_at(u0 - 2 * e_ * du, v0 - 2 * e_ * dv, lid - 2 * e_ * dl)
                fd4 = (8.0 * (Jp - Jm) - (J2p - J2m)) / (12 * e_)
            if e_ == eps:
                pairs.append((ad, fd))
                errs.append(abs(ad - fd) / max(abs(fd), 1e-300))
                if fd4 is not None:
                    errs4.append(abs(ad - fd4) / max(abs(fd4), 1e-300))
            else:
                sweep.setdefault(e_, []).append(
                    (abs(ad - fd) / max(abs(fd), 1e-300),
                     None if fd4 is None else abs(ad - fd4) / max(abs(fd4), 1e-300)))
    t_fd = time.perf_counter() - t0
    s.close()
    if rank != 0:
        return
    cells = case.cells
    cpu = None
    if not args.no_cpu_baseline:
        cv, csec, cores, kind, how = cpu_step_sample(case, (u0, v0, p0), 1)
        cpu = {"value": cv, "unit": UNIT, "cores": cores, "kind": kind,
               "sample": f"1 forward reference step of the same {n}x{n} case ({csec:.1f} s); {how}; the reference "
                         f"has no adjoint: one finite-difference gradient component costs two such {nsteps}-step runs"}
    line = {
        "metric": METRIC, "value": cells * nsteps / t_adj, "unit": UNIT, "n_gpus": 1,
        "steps": nsteps, "warmup": 0, "ms_per_step": 1e3 * t_adj / nsteps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": (
            (f"adjoint: lid-driven cavity {n}x{n}, Re={ADJOINT['re']:g}, dt={ADJOINT['dt']:g}, "
             f"{nsteps} steps from the seeded 16x16-mode perturbation (seed {args.seed}), rb_sor, "
             f"plain FP64; J = 0.5 h^2 sum(u^2+v^2) at the final step; gradient with respect to "
             f"the initial u, v, p and the {case.nx + 2}-value lid profile (256 moving-wall "
             f"positions), checkpoint every {every} steps, iteration counts of the forward run held fixed")
            if args.adj_case != "channel" else
            (f"adjoint: profiled channel {CHANNEL['ncx']}x{CHANNEL['ncy']} (mass-conserving outlet), "
             f"deck Re={CHANNEL['re']:g}, dt={CHANNEL['dt']:g}, {nsteps} steps (a reduced horizon of the "
             f"1000-step workload) from the flow after two steps, plain FP64; J = 0.5 h^2 sum(u^2+v^2) at "
             f"the final step; gradient with respect to the initial u, v, p and the {lid.size}-value inflow "
             f"profile, checkpoint every {every} steps, iteration counts held fixed")),
                   "value_is": "cell-steps of the forward horizon per second of the whole gradient "
                               "(forward with checkpoints + recompute + adjoint)"},
        "gradient_s": t_adj, "forward_s": t_fwd, "adjoint_over_forward": t_adj / t_fwd,
        "J": J, "fd_check": {"directions": args.fd_dirs, "eps": eps, "max_rel_err": max(errs) if errs else None,
                             "median_rel_err": float(np.median(errs)) if errs else None,
                             "order4_max_rel_err": max(errs4) if errs4 else None,
                             "order4_median_rel_err": float(np.median(errs4)) if errs4 else None,
                             "eps_sweep": {f"{e_:g}": {"order2_max_rel_err": max(x[0] for x in v),
                                                      "order4_max_rel_err": (max(x[1] for x in v)
                                                                             if v[0][1] is not None else None)}
                                           for e_, v in sweep.items()},
                             "pairs": pairs[:8], "seconds": t_fd},
        "iterations": {"nql_min": int(counts[:, 0].min()), "nql_max": int(counts[:, 0].max()),
                       "nsor_min": int(counts[:, 1].min()), "nsor_max": int(counts[:, 1].max())},
        "lid_grad_norm": float(np.linalg.norm(gl)),
        "e2e": {"value": cells * nsteps / t_adj, "unit": UNIT, "h2d_bytes_per_step": 3 * (nx + 2) * (ny + 2) * 8 / nsteps,
                "d2h_bytes_per_step": 3 * (nx + 2) * (ny + 2) * 8 / nsteps,
                "note": "the gradient call takes host fields in and returns host gradients; value already end to end"},
        "roofline": None,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)


ENSEMBLE = {"count": 256, "seed": 2024}


def ensemble_members(args):
    return deck.ensemble_cases(args.ens_count, seed=args.ens_seed, solver="rb_sor")


def ensemble_config(args, members, inner, graph):
    ns = [m.n for m in members]
    mixed = args.precision == "mixed"
    step = (f"mixed step ({inner} FP32 sweeps per refinement pass)" if mixed
            else "plain FP64 step (bit-identical per case to the case stepped alone)")
    return {
        "workload": (f"batched ensemble: {len(members)} lid-driven cavities, N cells per side drawn "
                     f"uniformly from {{64, 96, ..., 512}} and Re log-uniform in [100, 5000] "
                     f"(numpy default_rng({args.ens_seed})), dt = 0.5 h capped at the viscous number "
                     f"dt/(h^2 Re) = 0.25 where the reference scheme is unstable, seeded 16x16-mode "
                     f"streamfunction perturbation per case, rb_sor, {step}, one launch per stage for "
                     f"all cases"
                     f"{', step captured in a CUDA graph' if graph else ''}"),
        "cases": len(members), "cells": int(sum(m.case.cells for m in members)),
        "n_min": min(ns), "n_max": max(ns), "dt_capped_cases": sum(1 for m in members if m.dt < m.dt_named),
        "layout": "each cavity the unit square with h = 1/N; the Poisson rows of every member round to "
                  "the unit stencil in FP32 (exactly unit only for N a power of two)",
        "precision": args.precision, "graph": graph,
        "threads_per_block": args.ens_threads or 128, "sweeps_per_barrier": args.ens_k or 4,
        "l2": "not flushed: the ensemble's fields alone exceed L2 (129 MB) many times over",
    }


def run_ensemble(args):
    """The batched ensemble of 256 cavities: every case advanced together by one
    launch per stage; cases are spread over ranks by work, no exchange."""
    import torch
    import torch.distributed as dist
    from wolfd2_gb300 import replicas
    from wolfd2_gb300.gpu import PREC_FP64, PREC_MIXED, Ensemble, Solver

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    members = ensemble_members(args)
    mine = replicas.partition_work([m.case.cells for m in members], world, rank)
    graph = not args.no_graph
    inner = args.refine_sweeps or 64
    mixed = args.precision == "mixed"
    kw = {"refine_sweeps": inner, "precision": PREC_MIXED if mixed else PREC_FP64}
    solvers, ics = [], []
    for i in mine:
        c = members[i].case
        s = Solver.for_case(c, tuned=False)
        if args.no_tma:
            s.set_tma(False)
        ic = deck.perturbation_ic(c, args.seed + i)
        s.load_fields(*ic)
        solvers.append(s)
        ics.append(ic)
    ens = Ensemble(solvers, threads=args.ens_threads, sweeps_per_barrier=args.ens_k, graph=graph)
    prm = [members[i].case.params for i in mine]
    cells = sum(members[i].case.cells for i in mine)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    if args.warmup:
        ens.step(prm, args.warmup, **kw)
    # per-stage split of the same kind of steps (direct launches, events)
    ens.graph(False)
    ens.profile(True)
    prof_hist = ens.step(prm, 1, **kw)
    stages = ens.profile_read(mixed)
    ens.profile(False)
    ens.graph(graph)
    barrier()
    l0 = ens.info()["launches"]
    with ClockSampler(local) as clk:
        barrier()
        t0 = time.perf_counter()
        hist = ens.step(prm, args.steps, **kw)
        barrier()
        wall = time.perf_counter() - t0
    info = ens.info()
    t_dev = info["last_ms"] / 1e3
    launches = info["launches"] - l0
    # end to end: every step loads all fields from pinned host buffers,
    # steps, and reads them back
    pinned, hosts = [], []
    for s in solvers:
        ts = [torch.empty((s.mny + 1, s.mnx + 1), dtype=torch.float64, pin_memory=True) for _ in range(3)]
        hs = [t.numpy().T for t in ts]
        for h, f in zip(hs, s.store_fields()):
            h[...] = f
        pinned.append(ts)
        hosts.append(hs)
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    field_bytes = sum((s.mnx + 1) * (s.mny + 1) * 8 for s in solvers)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for s, hs in zip(solvers, hosts):
            s.load_fields(*hs)
        ens.step(prm, 1, **kw)
        for s, hs in zip(solvers, hosts):
            s.store_fields(out=hs)
    barrier()
    t_e2e = time.perf_counter() - t0
    tt = replicas.max_over_ranks((t_dev, t_e2e), device=dev)
    t_max, t_e2e_max = tt
    cells_all = sum(m.case.cells for m in members)
    if rank != 0:
        ens.close()
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return
    # algorithmic bytes of the dominant stage (the Poisson launch) over its
    # profiled step, summed over this rank's cases
    kname = "ke_ppe_mixed" if mixed else "ke_ppe"
    ppe_ms, _ = stages[kname]
    if mixed:
        alg = sum(mixed_ppe_bytes(members[i].case.cells, h[0][1], inner) for i, h in zip(mine, prof_hist))
    else:
        alg = sum(ppe_bytes(members[i].case.cells, h[0][1]) for i, h in zip(mine, prof_hist))
    peak_gbs, peak_kind = peaks()
    traffic_ratio = None
    try:
        traffic_ratio = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))[
            "bytes_per_alg_byte"].get(kname)
    except Exception:
        traffic_ratio = None
    achieved = alg / (ppe_ms / 1e3) / 1e9 if ppe_ms > 0 else None
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak_gbs,
            "unit": "GB/s", "frac": achieved / peak_gbs if achieved else None,
            "peak_kind": peak_kind,
            "traffic": traffic_ratio * alg if traffic_ratio else None,
            "alg_bytes_per_launch": alg, "avg_launch_ms": ppe_ms}
    cpu = None
    if not args.no_cpu_baseline:
        # a bounded sample: one reference step of the first cases in draw
        # order until about 15 s of host time
        done, secs, how, kind = 0, 0.0, "", "port"
        for i, m in enumerate(members):
            r, kind, how = reference_runner(m.case, deck.perturbation_ic(m.case, args.seed + i))
            t0 = time.perf_counter()
            r.step(1)
            secs += time.perf_counter() - t0
            done += m.case.cells
            if secs > 15.0:
                break
        cpu = {"value": done / secs, "unit": UNIT, "cores": 1, "kind": kind,
               "sample": f"1 reference step of each of the first {i + 1} cases ({done} cells, {secs:.1f} s); {how}"}
    nql = [h[0] for hh in hist for h in hh]
    nsor = [h[1] for hh in hist for h in hh]
    line = {
        "metric": METRIC, "value": cells_all * args.steps / t_max, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
        "steps_per_s": args.steps / t_max,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "f32+f64" if mixed else "f64", "data": "synthetic",
        "config": ensemble_config(args, members, inner, graph),
        "parallelism": f"cases partitioned by work over {world} ranks" if world > 1 else "single GPU",
        "roofline": roof,
        "e2e": {"value": cells_all * e2e_steps / t_e2e_max, "unit": UNIT,
                "h2d_bytes_per_step": 3 * field_bytes, "d2h_bytes_per_step": 3 * field_bytes,
                "steps": e2e_steps, "host_buffers": "pinned"},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": launches,
        "kernel_ms": {k: {"total_ms": v[0], "launches": v[1]} for k, v in stages.items()},
        "launch_blocks": {"momentum": info["blocks_momentum"], "poisson": info["blocks_poisson"]},
        "iterations": {"nql_min": min(nql), "nql_max": max(nql), "nsor_min": min(nsor), "nsor_max": max(nsor)},
        "divmax_max": max(h[3] for hh in hist for h in hh),
        "wall_s": wall,
    }
    print(json.dumps(line), flush=True)
    ens.close()
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["cavity", "channel", "ensemble", "adjoint", "thermal", "clustered"],
                    default="cavity",
                    help="cavity: the lid-driven cavity (--n cells per side); channel: the "
                         "4096x1024 plane channel with a profiled inflow; ensemble: 256 cavities "
                         "of uneven size and Re advanced together; thermal: the differentially "
                         "heated cavity with the energy equation (--n cells per side); clustered: "
                         "the lid-driven cavity on a wall-clustered Cartesian grid (--n cells per side)")
    ap.add_argument("--ens-count", type=int, default=ENSEMBLE["count"])
    ap.add_argument("--ens-seed", type=int, default=ENSEMBLE["seed"])
    ap.add_argument("--no-graph", action="store_true", help="ensemble: launch directly, no CUDA graph")
    ap.add_argument("--ens-threads", type=int, default=0, help="ensemble: threads per block (0: library default)")
    ap.add_argument("--ens-k", type=int, default=0, choices=[0, 4, 8],
                    help="ensemble: Poisson sweeps per grid barrier (0: library default)")
    ap.add_argument("--no-tma", action="store_true",
                    help="stage the several-tiles-per-block Poisson boxes with vector loads, not TMA")
    ap.add_argument("--adj-steps", type=int, default=ADJOINT["steps"], help="adjoint: steps of the horizon")
    ap.add_argument("--adj-case", choices=["cavity", "channel"], default="cavity",
                    help="adjoint: the 256x256 cavity (lid profile) or the profiled channel (inflow profile)")
    ap.add_argument("--fd-dirs", type=int, default=4, help="adjoint: finite-difference directions checked")
    ap.add_argument("--fd-eps", default="", help="adjoint: further eps values for the same directions, "
                    "comma-separated (eps=1e-6 is always checked)")
    ap.add_argument("--fd-order", type=int, choices=[2, 4], default=4,
                    help="adjoint: also check against the fourth-order central difference (4 runs per direction)")
    ap.add_argument("--n", type=int, default=1024, help="cavity cells per side")
    ap.add_argument("--re", type=float, default=1000.0)
    ap.add_argument("--dt", type=float, default=0.0,
                    help="time step (0: 2.5e-4; the clustered cavity 6.25e-5, the same CFL number on its "
                         "smallest cells, where 2.5e-4 drives the reference scheme to NaN)")
    ap.add_argument("--solver", default="rb_sor", choices=sorted(deck.PPE_SOLVERS))
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--sorrel", type=float, default=0.0,
                    help="sor_relaxation (0: the optimum 2/(1+sin(pi/n)) for the cavity, else 1)")
    ap.add_argument("--sortol", type=float, default=0.0, help="sor_tolerance (0: 1e-9 cavity, else 1e-8)")
    ap.add_argument("--msorit", type=int, default=0, help="max_sor_iter (0: 20000 cavity, else 2000)")
    ap.add_argument("--ppe-defaults", action="store_true",
                    help="the reference's default Poisson settings (sorrel 1, sortol 1e-8, 2000 sweeps)")
    ap.add_argument("--ref-seconds", type=float, default=100.0,
                    help="reference arm: time budget of its sample of whole steps")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--threads", type=int, default=0, help="threads per block (0: library default)")
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--seg", type=int, default=0, help="chain segment rows (0: auto)")
    ap.add_argument("--warm", type=int, default=0, help="chain warm-up rows (0: default)")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed",
                    help="headline path; mixed also times plain FP64 beside it")
    ap.add_argument("--refine-sweeps", type=int, default=0,
                    help="mixed: FP32 sweeps per refinement pass (0: 16 x sweeps per barrier)")
    ap.add_argument("--mixed-k", type=int, default=0, help="mixed: sweeps per grid barrier (4/8)")
    ap.add_argument("--mixed-threads", type=int, default=0, help="mixed: threads per block")
    ap.add_argument("--mixed-mode", type=int, default=0,
                    help="mixed: tile mode (0 auto, 1 several tiles per block, 3 two resident blocks per SM)")
    args = ap.parse_args()
    if not args.dt:
        args.dt = 6.25e-5 if args.workload == "clustered" else 2.5e-4
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "ensemble":
        run_ensemble(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
