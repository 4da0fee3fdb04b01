"""Generate the golden fixtures under tests/golden/: short time loops of the
oracle, each checked against the mechanical translation of the reference's
own Fortran source (oracle/f77ref.py) when the reference tree is present.

  cavity64_sor.json          64x64 lid-driven cavity, Re=100, dt=0.005,
                             point SOR, cold start, all 500 steps of the
                             configuration
  heated24_filter.json       24x24 differentially heated cavity (energy
                             equation, EqState, buoyancy), two momentum /
                             energy iterations, Filter of t, 6 steps
  thermal_multiregion.json   the curvilinear 3 x 2 region layout with a
                             fixed-temperature and a heat-generating region,
                             3 momentum / energy iterations, 5 steps
  curvilinear_rb_lsor.json   the curvilinear 3 x 2 layout, plain step,
                             lcartes = 0 (cross terms in every sweep),
                             red-black line SOR, 5 steps

Each file records which produced it: the oracle alone, or the translated
reference source with the oracle equal to it bit for bit.  Besides the
iteration counts, the last step's differences and the exact sums, it keeps
the SHA-256 of every final field's bytes ((nx+2) x (ny+2) doubles,
Fortran order), so a run matches a fixture only if every value matches."""
import hashlib
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(HERE)]

import f77ref  # noqa: E402
import oracle as O  # noqa: E402
import thermal_setup  # noqa: E402
from wolfd2_gb300 import deck  # noqa: E402


def _cavity64():
    return deck.cavity(64, 100.0, 0.005, solver="sor")


def _heated24():
    case = deck.heated_cavity(24, 500.0, 0.004, nmeiter=2, dmeittol=1e-7)
    case.tparams.nfiltt = 1
    case.tparams.fpt = 20.0
    return case


def _curvilinear_rb_lsor():
    case = thermal_setup.curvilinear_case()
    case.params.npsolver = deck.PPE_SOLVERS["rb_lsor"]
    case.params.msorit = 300
    return case


# name -> (case factory, steps, description, fields)
FIXTURES = {
    "cavity64_sor": (_cavity64, 500, "cavity 64x64, Re=100, dt=0.005, ppe_solver sor, cold start",
                     "uvp"),
    "heated24_filter": (_heated24, 6, "heated cavity 24x24, Re=500, Pr=0.71, Fr=0.05, dt=0.004, "
                        "nmeiter 2, EqState + buoyancy, filter_t 20, rb_sor", "uvptd"),
    "thermal_multiregion": (lambda: thermal_setup.loop_case(), 5,
                            "curvilinear 3 x 2 regions, fixed-temperature and heat-generating "
                            "regions, energy equation with EqState and buoyancy", "uvptd"),
    "curvilinear_rb_lsor": (_curvilinear_rb_lsor, 5, "curvilinear 3 x 2 regions, lcartes 0, "
                            "ppe_solver rb_lsor, msorit 300", "uvp"),
}


def field_hash(a, nx, ny):
    """SHA-256 of the (0:nx+1, 0:ny+1) part of a field, Fortran order."""
    return hashlib.sha256(np.asfortranarray(a[:nx + 2, :ny + 2]).tobytes(order="F")).hexdigest()


def summary(o, fields, nx, ny):
    """The record a fixture keeps of a run."""
    out = {"cold_nconv": o.cold_nconv,
           "iterations": [[h[0], h[1]] for h in o.history],
           "dif_last": list(o.history[-1][2]),
           "sum": {k: math.fsum(o.f[k].ravel()) for k in fields},
           "abs_sum": {k: math.fsum(np.abs(o.f[k]).ravel()) for k in fields},
           "sha256": {k: field_hash(o.f[k], nx, ny) for k in fields}}
    return out


def make(name):
    factory, steps, desc, fields = FIXTURES[name]
    case = factory()
    o = O.OracleRun(case)
    o.step(steps)
    src = "oracle"
    if f77ref.available():
        import refrun
        f77ref.build(case.nx + 1, case.ny + 1)
        r = refrun.RefRun(case)
        r.step(steps)
        for k in fields:
            assert np.array_equal(r.f[k], o.f[k]), (name, k)
        assert [h[:2] for h in r.history] == [h[:2] for h in o.history], name
        assert [h[2] for h in r.history] == [h[2] for h in o.history], name
        src = "translated reference source (oracle/f77ref.py), equal to the oracle"
    out = {"case": desc, "steps": steps, "source": src}
    out.update(summary(o, fields, case.nx, case.ny))
    out["fields"] = fields
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        f.write(json.dumps(out, indent=1, separators=(",", ": "))
                .replace("[\n   ", "[").replace(",\n   ", ", ").replace("\n  ]", "]"))
    print("wrote", name, "from", out["source"])


def main():
    for name in (sys.argv[1:] or FIXTURES):
        make(name)


if __name__ == "__main__":
    main()
