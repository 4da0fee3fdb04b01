"""Time loop over the mechanically translated reference routines (TEST
INFRASTRUCTURE ONLY).

The routines come from oracle/f77ref.py's translation of the reference
source; this module only sequences them exactly as the reference's main
program does for nthermen = nsmallscl = 0 (src/main.f:606-641 cold start,
src/main.f:690-972 one time step), using the reference's own argument names.
"""
from __future__ import annotations

from typing import Dict, Optional

import numpy as np

import f77ref

METRICS = ("ran rbn rgn rac rbc rgc rau rbu rbv rgv dju djv djc djn "
           "xen yen xzn yzn xec yec xzc yzc xeu yeu xzv yzv xzu yzu xev yev").split()


class RefRun:
    def __init__(self, case, fields: Optional[Dict[str, np.ndarray]] = None, cold_start: bool = True):
        self.case = case
        self.nx, self.ny = case.nx, case.ny
        self.mnx, self.mny = case.nx + 1, case.ny + 1
        self.R = f77ref.RefLib(self.mnx, self.mny)
        z = lambda: np.zeros((self.mnx + 1, self.mny + 1), np.float64, order="F")  # noqa: E731
        self.z = z
        reg = case.regions
        self.tab = dict(nreg=np.ascontiguousarray(reg.nReg, np.int32),
                        nregbrd=np.asfortranarray(reg.nRegBrd, np.int32),
                        nregtype=np.asfortranarray(reg.nRegType, np.int32),
                        nmombdtp=np.asfortranarray(reg.nMomBdTp, np.int32),
                        dbcval=np.asfortranarray(reg.dBCVal),
                        dprporos=np.asfortranarray(reg.dPRporos),
                        dprporc1=np.asfortranarray(reg.dPRporc1),
                        dprporc2=np.asfortranarray(reg.dPRporc2))
        # Grid: MirrorPts, FullGrid, Metric (src/grid.f:105-124)
        x, y = z(), z()
        x[1:self.nx + 1, 1:self.ny + 1] = case.x
        y[1:self.nx + 1, 1:self.ny + 1] = case.y
        self.m = {k: z() for k in METRICS}
        xu, yu, xv, yv, xc, yc = (z() for _ in range(6))
        n = dict(nx=self.nx, ny=self.ny)
        self.R("mirrorpts", **n, x=x, y=y)
        self.R("fullgrid", **n, x=x, y=y, xu=xu, yu=yu, xv=xv, yv=yv, xc=xc, yc=yc)
        self.R("metric", **n, xn=x, yn=y, xu=xu, yu=yu, xv=xv, yv=yv, xc=xc, yc=yc, **self.m)
        self.f = {k: z() for k in "u v p t un vn pn tn us vs ts d dn".split()}
        if fields:
            for k, v in fields.items():
                self.f[k][...] = v
        self.history = []
        self.cold_nconv = None
        if cold_start:
            self.cold_nconv = self._cold_start()

    # -- wrappers with the reference's argument names --------------------
    def vel_bc(self, u, v):
        t = self.tab
        self.R("velboundcond", nx=self.nx, ny=self.ny, nreg=t["nreg"], nregbrd=t["nregbrd"],
               nmombdtp=t["nmombdtp"], dbcval=t["dbcval"], u=u, v=v)

    def pres_bc(self, p):
        t = self.tab
        self.R("presboundcond", nx=self.nx, ny=self.ny, nreg=t["nreg"], nregbrd=t["nregbrd"],
               nregtype=t["nregtype"], nmombdtp=t["nmombdtp"], dbcval=t["dbcval"], p=p)

    def ppe(self, u, v, p, npsolver=None, msorit=None) -> int:
        prm, t, m = self.case.params, self.tab, self.m
        _, outs = self.R("ppe", nx=self.nx, ny=self.ny, nreg=t["nreg"], nregbrd=t["nregbrd"],
                         nregtype=t["nregtype"], lcartesgrid=prm.lcartes,
                         nppesolver=prm.npsolver if npsolver is None else npsolver,
                         msorit=prm.msorit if msorit is None else msorit, nsorconv=0,
                         dk=prm.dk, sortol=prm.sortol, sorrel=prm.sorrel,
                         rau=m["rau"], rbu=m["rbu"], rbv=m["rbv"], rgv=m["rgv"],
                         xeu=m["xeu"], yeu=m["yeu"], xzv=m["xzv"], yzv=m["yzv"], u=u, v=v, p=p)
        return outs["nsorconv"]

    def project(self, p, u, v):
        t, m = self.tab, self.m
        self.R("project", nx=self.nx, ny=self.ny, nreg=t["nreg"], nregbrd=t["nregbrd"],
               nregtype=t["nregtype"], nmombdtp=t["nmombdtp"], dk=self.case.params.dk,
               dju=m["dju"], djv=m["djv"], yeu=m["yeu"], xzv=m["xzv"], yzu=m["yzu"],
               xev=m["xev"], p=p, u=u, v=v)

    def naux(self, un, vn, us, vs) -> int:
        prm, t, m, f = self.case.params, self.tab, self.m, self.f
        r, _ = self.R("nauxmomentum", nx=self.nx, ny=self.ny, mqiter=prm.mqiter,
                      nreg=t["nreg"], nregbrd=t["nregbrd"], nregtype=t["nregtype"],
                      nmombdtp=t["nmombdtp"], dk=prm.dk, re=prm.re, fr=prm.fr, qtol=prm.qtol,
                      dprporos=t["dprporos"], dprporc1=t["dprporc1"], dprporc2=t["dprporc2"],
                      dbcval=t["dbcval"], d=f["d"], dn=f["dn"], un=un, vn=vn, us=us, vs=vs,
                      **{k: m[k] for k in ("ran", "rbn", "rgn", "rac", "rbc", "rgc", "dju", "djv",
                                           "xec", "yec", "xzn", "yzn", "xen", "yen", "xzc", "yzc",
                                           "xeu", "yeu", "xzu", "yzu", "xev", "yev", "xzv", "yzv")})
        return int(r)

    def diff(self, a, b) -> float:
        r, _ = self.R("diffmaxnorm", nx=self.nx, ny=self.ny, un=a, u=b)
        return float(r)

    # -- main.f ------------------------------------------------------------
    def _cold_start(self) -> int:
        f = self.f
        self.vel_bc(f["u"], f["v"])
        n = self.ppe(f["u"], f["v"], f["p"])
        self.pres_bc(f["p"])
        self.project(f["p"], f["u"], f["v"])
        self.vel_bc(f["u"], f["v"])
        return n

    def step(self, n: int = 1):
        f = self.f
        for _ in range(n):
            for a, b in (("pn", "p"), ("un", "u"), ("vn", "v"), ("tn", "t"), ("dn", "d")):
                f[a][...] = f[b]
            for a, b in (("us", "u"), ("vs", "v"), ("ts", "t")):
                f[a][...] = f[b]
            nql = self.naux(f["un"], f["vn"], f["us"], f["vs"])
            self.vel_bc(f["us"], f["vs"])
            self.pres_bc(f["p"])
            nsor = self.ppe(f["us"], f["vs"], f["p"])
            self.pres_bc(f["p"])
            self.project(f["p"], f["us"], f["vs"])
            self.vel_bc(f["us"], f["vs"])
            self.pres_bc(f["p"])
            for a, b in (("u", "us"), ("v", "vs"), ("t", "ts")):
                f[a][...] = f[b]
            self.vel_bc(f["u"], f["v"])
            self.pres_bc(f["p"])
            dif = (self.diff(f["pn"], f["p"]), self.diff(f["un"], f["u"]),
                   self.diff(f["vn"], f["v"]), self.diff(f["tn"], f["t"]))
            self.history.append((nql, nsor, dif))
        return self.history[-1]
