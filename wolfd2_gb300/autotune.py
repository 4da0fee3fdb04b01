"""Autotuner of the kernel shapes, per grid shape and precision.

The tuned knobs change only how the work is laid out on the GPU, never the
arithmetic: every setting gives bit-identical results (the chain solves are
exact for any segment length and warm-up; the mixed Poisson sweeps give the
same bits for any tile shape and sweeps-per-barrier), except the mixed path's
FP32 sweeps per refinement pass, which sets how often the FP64 residual is
re-formed and is therefore searched only over values whose accuracy the tests
cover (64-256).

    python -m wolfd2_gb300.autotune --n 1024 --n 512 [--precision mixed]
    python -m wolfd2_gb300.autotune --channel 4096x1024

times every candidate on the current GPU (device time of a few steps of the
seeded-perturbation cavity, or of the profiled channel from its initial
field, CUDA events through the library's profiler) and merges the fastest
into ``tuned.json`` beside this file.  ``Solver.for_case`` applies the entry
of its grid shape when one exists.
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
from typing import Dict, Optional

HERE = os.path.dirname(os.path.abspath(__file__))
TUNED = os.path.join(HERE, "tuned.json")

CHAIN_SEG = (0, 16, 32, 48, 128, 512)   # 0: the library's default (rows / threads)
CHAIN_WARM = (24, 48, 64)
MIXED_K = (4, 8)
MIXED_THREADS = (256, 384, 512)
MIXED_MODE = (0, 1, 3)            # 0: resident tiles when they fit, 1: multi-tile, 3: two resident tiles per SM
REFINE = (64, 128, 256)


def key(nx: int, ny: int, precision: str) -> str:
    return f"{nx}x{ny}:{precision}"


def load() -> Dict[str, dict]:
    if os.path.exists(TUNED):
        with open(TUNED) as f:
            return json.load(f)
    return {}


def lookup(nx: int, ny: int, precision: str) -> Optional[dict]:
    return load().get(key(nx, ny, precision))


def apply(solver, cfg: Optional[dict]) -> None:
    """Set a tuned configuration on a Solver (None: leave the defaults)."""
    if not cfg:
        return
    solver.tune(seg=cfg.get("seg", 0), warm=cfg.get("warm", 0))
    if cfg.get("mixed_k") or cfg.get("mixed_threads"):
        try:
            solver.tune_mixed(cfg.get("mixed_k", 0), cfg.get("mixed_threads", 0), cfg.get("mixed_mode", 0))
        except Exception:  # a shape the mixed planner rejects: keep its default
            pass
    solver.refine_sweeps = cfg.get("refine_sweeps", 0)


def _time(solver, case, fields, precision: int, refine: int, steps: int) -> float:
    """Device ms per step of `steps` steps after one warm-up step."""
    from .gpu import K_BC, K_COPY, K_MOMENTUM, K_POST, K_PPE
    prm = case.params
    solver.load_fields(*fields)
    solver.step(prm, 1, precision=precision, refine_sweeps=refine)
    solver.profile(True)
    solver.step(prm, steps, precision=precision, refine_sweeps=refine)
    ms = sum(solver.profile_read(k)[0] for k in (K_MOMENTUM, K_PPE, K_POST, K_BC, K_COPY))
    solver.profile(False)
    return ms / steps


def tune_case(case, precision: str = "mixed", steps: int = 2, seed: int = 1234, log=print,
              fields=None) -> dict:
    """Coordinate search: chain segment shape first, then (mixed) the Poisson
    kernel shape, tile mode and the refinement pass length."""
    from . import deck
    from .gpu import PREC_FP64, PREC_MIXED, Solver, W2Error
    prec = PREC_MIXED if precision == "mixed" else PREC_FP64
    s = Solver.for_case(case, tuned=False)
    if fields is None:
        fields = deck.perturbation_ic(case, seed)
    best = {"seg": 0, "warm": 64, "mixed_k": 8 if prec == PREC_MIXED else 0,
            "mixed_threads": 512 if prec == PREC_MIXED else 0, "mixed_mode": 0,
            "refine_sweeps": 128 if prec == PREC_MIXED else 0}

    def run(cfg):
        apply(s, cfg)
        try:
            return _time(s, case, fields, prec, cfg["refine_sweeps"], steps)
        except W2Error as e:
            log(f"  {cfg}: {e}")
            return float("inf")

    best_ms = run(best)
    log(f"start {best} {best_ms:.3f} ms/step")
    for seg, warm in itertools.product(CHAIN_SEG, CHAIN_WARM):
        cfg = {**best, "seg": seg, "warm": warm}
        ms = run(cfg)
        log(f"  chain {seg:4d} {warm:3d}: {ms:.3f}")
        if ms < best_ms:
            best, best_ms = cfg, ms
    if prec == PREC_MIXED:
        for k, t, mode, r in itertools.product(MIXED_K, MIXED_THREADS, MIXED_MODE, REFINE):
            cfg = {**best, "mixed_k": k, "mixed_threads": t, "mixed_mode": mode, "refine_sweeps": r}
            ms = run(cfg)
            log(f"  mixed K={k} threads<={t} mode={mode} inner={r}: {ms:.3f}")
            if ms < best_ms:
                best, best_ms = cfg, ms
    best["ms_per_step"] = best_ms
    log(f"best {best}")
    s.close()
    return best


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--n", type=int, action="append", help="cavity cells per side (repeatable)")
    ap.add_argument("--channel", action="append", metavar="NCXxNCY",
                    help="profiled channel cells, e.g. 4096x1024 (Re 1e4, dt 2.5e-4; repeatable)")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--re", type=float, default=1000.0)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--out", default=TUNED)
    args = ap.parse_args()
    from . import deck
    table = load() if os.path.abspath(args.out) == TUNED else {}
    if os.path.exists(args.out):
        with open(args.out) as f:
            table.update(json.load(f))
    jobs = []
    for n in args.n or ([] if args.channel else [1024]):
        jobs.append((deck.cavity(n, args.re, 0.25 / n, solver="rb_sor"), None))
    for spec in args.channel or []:
        ncx, ncy = (int(t) for t in spec.lower().split("x"))
        case = deck.channel_inflow(ncx, ncy, 1.0e4, 2.5e-4)
        jobs.append((case, deck.channel_ic(case)))
    for case, fields in jobs:
        cfg = tune_case(case, args.precision, args.steps, fields=fields)
        table[key(case.nx, case.ny, args.precision)] = cfg
        with open(args.out, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
