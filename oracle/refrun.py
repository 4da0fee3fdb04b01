"""Time loop over the mechanically translated reference routines (TEST
INFRASTRUCTURE ONLY).

The routines come from oracle/f77ref.py's translation of the reference
source; this module only sequences them exactly as the reference's main
program does for nsmallscl = 0 (src/main.f:606-641 cold start,
src/main.f:690-972 one time step, with the momentum/energy iterations when
the case carries thermal parameters), using the reference's own argument
names.
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
        self.atd = getattr(case, "atd", None)
        if self.atd is not None:
            for k in ("uss", "vss", "pss", "tss", "usn", "vsn", "tsn"):
                self.f[k] = z()
            self.small_scale(0)   # main.f:645-664

    def small_scale(self, initflg):
        """SmallScale(initflg) on the fields u, v, t (main.f:645-664, 911-930)."""
        a, p, tb, m, f = self.atd, self.case.params, self.tab, self.m, self.f
        tt = self._ttab()
        self.R("smallscale", nx=self.nx, ny=self.ny, initflg=initflg, nthermen=0,
               lcartesgrid=p.lcartes, nreg=tb["nreg"], nregbrd=tb["nregbrd"], nregtype=tb["nregtype"],
               ntrgtype=tt["ntrgtype"], nmombdtp=tb["nmombdtp"], ntembdtp=tt["ntembdtp"],
               nppesolver=a.npsolver, msorit=a.msorit, dlref=a.dlref, uref=a.uref, tref=a.tref,
               tmax=a.tmax, dka=p.dk, re=p.re, pe=a.pe, sortol=a.sortol, sorrel=a.sorrel,
               fp=np.array([a.fpu, a.fpv, 0.0, a.fpt]), cu0=a.cu0, tscoef=a.tscoef,
               hscoef=a.hscoef, temcoef=a.temcoef, bnumc=a.bnumc, rmax=a.rmax, rlc=a.rlc,
               dtrgval=tt["dtrgval"], dbcval=tb["dbcval"],
               **{k: m[k] for k in ("rau", "rbu", "rbv", "rgv", "dju", "djv", "djc", "xeu", "yeu",
                                    "xzv", "yzv", "xzu", "yzu", "xev", "yev", "xec", "yec", "xzc",
                                    "yzc")},
               u1=f["u"], v1=f["v"], t1=f["t"], uss=f["uss"], vss=f["vss"], pss=f["pss"],
               tss=f["tss"])

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

    # -- thermal (case.thermal: deck.Thermal, case.tparams: deck.ThermalParams)
    def _ttab(self):
        th = self.case.thermal
        if th is None:
            from wolfd2_gb300.deck import Thermal
            th = Thermal.empty()
        return dict(ntrgtype=np.asfortranarray(th.nTRgType, np.int32),
                    ntembdtp=np.asfortranarray(th.nTemBdTp, np.int32),
                    dtrgval=np.asfortranarray(th.dTRgVal, np.float64))

    def temp_bc(self, t):
        tb = self.tab
        self.R("tempboundcond", nx=self.nx, ny=self.ny, nreg=tb["nreg"], nregbrd=tb["nregbrd"],
               **self._ttab(), dbcval=tb["dbcval"], t=t)

    def therm(self, un, vn, u, v, tn, t):
        tb, m, tp = self.tab, self.m, self.case.tparams
        self.R("thermenergy", nx=self.nx, ny=self.ny, nreg=tb["nreg"], nregbrd=tb["nregbrd"],
               **self._ttab(), dhgstval=np.asfortranarray(self.case.thermal.dHGSTval, np.float64),
               dk=self.case.params.dk, pe=tp.pe, dbcval=tb["dbcval"],
               **{k: m[k] for k in ("rau", "rbu", "rbv", "rgv", "djc", "xeu", "yeu", "xzv", "yzv",
                                    "xec", "yec", "xzc", "yzc")},
               un=un, vn=vn, u=u, v=v, tn=tn, t=t)

    def eq_state(self, p, t, den):
        tp = self.case.tparams
        self.R("eqstate", nx=self.nx, ny=self.ny, uref=tp.uref, densref=tp.densref, tmax=tp.tmax,
               tref=tp.tref, rconst=tp.rconst, p=p, t=t, den=den)

    def step(self, n: int = 1):
        """main.f:690-972: with case.tparams.nthermen = 1 the momentum/energy
        iterations (main.f:736-879) run ThermEnergy and EqState."""
        f = self.f
        tp = getattr(self.case, "tparams", None)
        therm = tp is not None and tp.nthermen == 1
        eqs = tp is not None and tp.neqstate == 1
        nme = tp.nmeiter if tp is not None else 1
        if not therm and nme > 0:
            nme = 1
        for _ in range(n):
            for a, b in (("pn", "p"), ("un", "u"), ("vn", "v"), ("tn", "t"), ("dn", "d")):
                f[a][...] = f[b]
            if self.atd is not None:   # main.f:708-730
                for a, b in (("usn", "uss"), ("vsn", "vss"), ("tsn", "tss")):
                    f[a][...] = f[b]
                for a, b in (("un", "uss"), ("vn", "vss"), ("tn", "tss")):
                    f[a][...] = f[a] + f[b]
            for l in range(1, nme + 1):
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
                if therm:
                    self.therm(f["un"], f["vn"], f["us"], f["vs"], f["tn"], f["ts"])
                if eqs:
                    self.eq_state(f["p"], f["ts"], f["d"])
                me = (self.diff(f["u"], f["us"]), self.diff(f["v"], f["vs"]), self.diff(f["t"], f["ts"]))
                for a, b in (("u", "us"), ("v", "vs"), ("t", "ts")):
                    f[a][...] = f[b]
                mx = me[0]
                for x in me[1:]:
                    mx = x if x > mx else mx
                if l > 1 and mx < tp.dmeittol:
                    break
            if therm and tp.nfiltt == 1:
                tb = self.tab
                self.R("filter", nx=self.nx, ny=self.ny, ncomp=4, nreg=tb["nreg"], nregbrd=tb["nregbrd"],
                       nregtype=tb["nregtype"], nmombdtp=tb["nmombdtp"],
                       ntrgtype=self._ttab()["ntrgtype"], fp=tp.fpt, qu=f["t"])
            if self.atd is not None:   # main.f:898-940
                for a, b in (("u", "usn"), ("v", "vsn"), ("t", "tsn")):
                    f[a][...] = f[a] - f[b]
                self.small_scale(1)
                for a, b in (("u", "uss"), ("v", "vss"), ("t", "tss")):
                    f[a][...] = f[a] + f[b]
            self.vel_bc(f["u"], f["v"])
            self.pres_bc(f["p"])
            if therm:
                self.temp_bc(f["t"])
            dif = (self.diff(f["pn"], f["p"]), self.diff(f["un"], f["u"]),
                   self.diff(f["vn"], f["v"]), self.diff(f["tn"], f["t"]))
            self.history.append((nql, nsor, dif))
        return self.history[-1] if self.history else None
