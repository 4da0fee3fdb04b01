"""Generate tests/golden/cavity64_sor.json: the first 40 steps of the 64x64
lid-driven cavity (Re=100, dt=0.005, point SOR, cold start).

The fixture is produced by the mechanical translation of the reference's own
Fortran source (oracle/f77ref.py) when the reference tree is present, and
must agree with the oracle (the script asserts it); the file records which
produced it."""
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

import f77ref  # noqa: E402
import oracle as O  # noqa: E402
from wolfd2_gb300 import deck  # noqa: E402

STEPS = 40


def main():
    case = deck.cavity(64, 100.0, 0.005, solver="sor")
    o = O.OracleRun(case)
    o.step(STEPS)
    src = "oracle"
    if f77ref.available():
        import refrun
        f77ref.build(case.nx + 1, case.ny + 1)
        r = refrun.RefRun(case)
        r.step(STEPS)
        for k in "uvp":
            assert np.array_equal(r.f[k], o.f[k]), k
        assert [h[:2] for h in r.history] == [h[:2] for h in o.history]
        src = "translated reference source (oracle/f77ref.py), equal to the oracle"
    out = {"case": "cavity 64x64, Re=100, dt=0.005, ppe_solver sor, cold start",
           "steps": STEPS, "source": src, "cold_nconv": o.cold_nconv,
           "iterations": [[h[0], h[1]] for h in o.history],
           "dif_last": list(o.history[-1][2]),
           "sum": {k: math.fsum(o.f[k].ravel()) for k in "uvp"},
           "abs_sum": {k: math.fsum(np.abs(o.f[k]).ravel()) for k in "uvp"}}
    with open(os.path.join(HERE, "cavity64_sor.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", out["source"])


if __name__ == "__main__":
    main()
