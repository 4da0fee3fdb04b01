"""The time loop with the small-scale model (nsmallscl = 1) driven from the
host through the drop-in entry points, as the Fortran driver calls them.

main.f seeds the small scales after the cold start (main.f:645-664), adds
the small scales of level n to the time-level copies before the momentum
update (main.f:708-730), and after the step removes them from the new
level, recomputes them with SmallScale from the large scales and adds them
back (main.f:898-940).  Every routine here is the library's device
drop-in; the additions and copies are the driver's own array statements.
This is the reference's calling pattern (one host round trip per routine),
not a throughput path: the device-resident loop (Solver.step) does not run
the small-scale model.
"""
from __future__ import annotations

from typing import Optional

import numpy as np

from .deck import Case, Thermal


class AtdLoop:
    """A case advanced by main.f's loop with SmallScale, on host arrays."""

    def __init__(self, solver, case: Case, fields: dict, ap, th: Optional[Thermal] = None,
                 tparams=None):
        self.s, self.case, self.ap = solver, case, ap
        self.th = th if th is not None else Thermal.empty()
        self.tp = tparams
        shape = (solver.mnx + 1, solver.mny + 1)
        z = lambda: np.zeros(shape, order="F")  # noqa: E731
        self.f = {k: z() for k in ("u", "v", "p", "t", "d", "un", "vn", "pn", "tn", "dn", "us", "vs", "ts",
                                   "uss", "vss", "pss", "tss", "usn", "vsn", "tsn")}
        for k, val in fields.items():
            self.f[k][...] = val
        self.history = []
        f = self.f
        # main.f:645-664: the small scales of the initial fields
        self.nsor_seed = solver.SmallScale(0, self.th, ap, f["u"], f["v"], f["t"], f["uss"], f["vss"],
                                           f["pss"], f["tss"])

    def step(self, n: int = 1):
        s, prm, f, tp = self.s, self.case.params, self.f, self.tp
        therm = tp is not None and tp.nthermen == 1
        eqs = tp is not None and tp.neqstate == 1
        nme = tp.nmeiter if (tp is not None and therm) else 1
        for _ in range(n):
            for a, b in (("pn", "p"), ("un", "u"), ("vn", "v"), ("tn", "t"), ("dn", "d")):
                f[a][...] = f[b]
            for a, b in (("usn", "uss"), ("vsn", "vss"), ("tsn", "tss")):
                f[a][...] = f[b]
            f["un"] += f["uss"]
            f["vn"] += f["vss"]
            f["tn"] += f["tss"]
            nql = nsor = 0
            for l in range(1, nme + 1):
                f["us"][...] = f["u"]
                f["vs"][...] = f["v"]
                f["ts"][...] = f["t"]
                nql = s.nAuxMomentum(prm.mqiter, prm.dk, prm.re, prm.fr, prm.qtol,
                                     f["d"] if eqs else None, f["dn"] if eqs else None,
                                     f["un"], f["vn"], f["us"], f["vs"])
                if prm.nfiltu == 1:
                    s.Filter(1, prm.fpu, f["us"])
                if prm.nfiltv == 1:
                    s.Filter(2, prm.fpv, f["vs"])
                s.VelBoundCond(f["us"], f["vs"])
                s.PresBoundCond(f["p"])
                nsor = s.Ppe(prm.lcartes, prm.npsolver, prm.msorit, prm.dk, prm.sortol, prm.sorrel,
                             f["us"], f["vs"], f["p"])
                s.PresBoundCond(f["p"])
                s.Project(prm.dk, f["p"], f["us"], f["vs"])
                s.VelBoundCond(f["us"], f["vs"])
                s.PresBoundCond(f["p"])
                if therm:
                    s.ThermEnergy(self.th, prm.dk, tp.pe, f["un"], f["vn"], f["us"], f["vs"], f["tn"], f["ts"])
                if eqs:
                    s.EqState(tp.uref, tp.densref, tp.tmax, tp.tref, tp.rconst, f["p"], f["ts"], f["d"])
                me = (s.DiffMaxNorm(f["u"], f["us"]), s.DiffMaxNorm(f["v"], f["vs"]),
                      s.DiffMaxNorm(f["t"], f["ts"]))
                f["u"][...] = f["us"]
                f["v"][...] = f["vs"]
                f["t"][...] = f["ts"]
                if l > 1 and max(me) < tp.dmeittol:
                    break
            if therm and tp.nfiltt == 1:
                s.FilterT(self.th, tp.fpt, f["t"])
            f["u"] -= f["usn"]
            f["v"] -= f["vsn"]
            f["t"] -= f["tsn"]
            s.SmallScale(1, self.th, self.ap, f["u"], f["v"], f["t"], f["uss"], f["vss"], f["pss"], f["tss"])
            f["u"] += f["uss"]
            f["v"] += f["vss"]
            f["t"] += f["tss"]
            s.VelBoundCond(f["u"], f["v"])
            s.PresBoundCond(f["p"])
            if therm:
                s.TempBoundCond(self.th, f["t"])
            dif = (s.DiffMaxNorm(f["pn"], f["p"]), s.DiffMaxNorm(f["un"], f["u"]),
                   s.DiffMaxNorm(f["vn"], f["v"]), s.DiffMaxNorm(f["tn"], f["t"]))
            self.history.append((nql, nsor, dif))
            if max(dif) > 1.0e12:
                raise FloatingPointError("Solution diverged. Please reduce CFL number.")
        return self.history[-1] if self.history else None
