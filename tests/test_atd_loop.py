"""The host side of the small-scale time loop (wolfd2_gb300.atd.AtdLoop:
main.f's loop with nsmallscl = 1, main.f:645-664, 708-730, 898-940) checked
on the CPU: driven by the oracle's routines under the drop-in names, it
reproduces the oracle's own loop (w2o_step_atd) bit for bit.  The device
drop-ins behind the same names are checked against the oracle routine by
routine in the GPU tests."""
import types

import numpy as np
import pytest

import oracle as O
from wolfd2_gb300 import deck
from wolfd2_gb300.atd import AtdLoop


class _OracleDropins:
    """The drop-in routine names AtdLoop calls, on one oracle context (the
    loop's routines and SmallScale share its saved arrays, as they share the
    reference's)."""

    def __init__(self, case):
        self.c = case
        self.o = O.Oracle(case.nx + 1, case.ny + 1)
        self.mnx, self.mny = self.o.mnx, self.o.mny
        self.met = self.o.grid(case.nx, case.ny, case.x, case.y)
        self.atd = None

    def SmallScale(self, initflg, th, ap, u, v, t, uss, vss, pss, tss):
        if self.atd is None:
            self.atd = O.SmallScale(self.o, self.c.nx, self.c.ny, self.c.regions, th, self.met, ap)
        return self.atd(initflg, u, v, t, uss, vss, pss, tss)

    def nAuxMomentum(self, mqiter, dk, re, fr, qtol, d, dn, un, vn, us, vs):
        prm = types.SimpleNamespace(mqiter=mqiter, dk=dk, re=re, fr=fr, qtol=qtol)
        z = self.o.field()
        return self.o.naux_momentum(self.c.nx, self.c.ny, self.c.regions, prm, self.met,
                                    z if d is None else d, z if dn is None else dn, un, vn, us, vs)

    def Filter(self, ncomp, fp, q):
        self.o.filter(self.c.nx, self.c.ny, ncomp, self.c.regions, fp, q)

    def VelBoundCond(self, u, v):
        self.o.vel_bound_cond(self.c.nx, self.c.ny, self.c.regions, u, v)

    def PresBoundCond(self, p):
        self.o.pres_bound_cond(self.c.nx, self.c.ny, self.c.regions, p)

    def Ppe(self, lcartes, npsolver, msorit, dk, sortol, sorrel, u, v, p):
        prm = types.SimpleNamespace(lcartes=lcartes, dk=dk, sortol=sortol, sorrel=sorrel)
        return self.o.ppe(self.c.nx, self.c.ny, self.c.regions, prm, self.met, u, v, p,
                          npsolver=npsolver, msorit=msorit)

    def Project(self, dk, p, u, v):
        self.o.project(self.c.nx, self.c.ny, self.c.regions, dk, self.met, p, u, v)

    def DiffMaxNorm(self, a, b):
        return self.o.diff_max_norm(self.c.nx, self.c.ny, a, b)

    def ThermEnergy(self, th, dk, pe, un, vn, u, v, tn, t):
        self.o.therm_energy(self.c.nx, self.c.ny, self.c.regions, th, dk, pe, self.met, un, vn, u, v, tn, t)

    def EqState(self, uref, densref, tmax, tref, rconst, p, t, den):
        self.o.eq_state(self.c.nx, self.c.ny, uref, densref, tmax, tref, rconst, p, t, den)

    def FilterT(self, th, fp, q):
        self.o.filter_t(self.c.nx, self.c.ny, self.c.regions, th, fp, q)

    def TempBoundCond(self, th, t):
        self.o.temp_bound_cond(self.c.nx, self.c.ny, self.c.regions, th, t)


@pytest.mark.parametrize("cu0,bnumc", [(0.0, 200.0), (2.0, 200.0), (2.0, 5.0)])
def test_atd_loop_calling_sequence(cu0, bnumc):
    case = deck.cavity(24, 800.0, 0.004, solver="rb_sor")
    dev = O.OracleRun(case)
    dev.step(30)
    fields = {k: dev.f[k].copy(order="F") for k in ("u", "v", "p", "t", "d")}
    case.atd = deck.SmallScaleParams(cu0=cu0, bnumc=bnumc, npsolver=deck.PPE_SOLVERS["rb_sor"], msorit=400,
                                     sorrel=1.3, fpu=300.0, fpv=300.0, fpt=200.0, pe=560.0)
    ref = O.OracleRun(case, fields=fields, cold_start=False)
    loop = AtdLoop(_OracleDropins(case), case, fields, ref._ap)
    assert loop.nsor_seed == ref.atd_nsor[0]
    ref.step(3)
    loop.step(3)
    assert [h[:2] for h in loop.history] == [h[:2] for h in ref.history]
    assert [tuple(h[2]) for h in loop.history] == [tuple(h[2]) for h in ref.history]
    for k in ("u", "v", "p", "t", "uss", "vss", "pss", "tss"):
        assert np.array_equal(loop.f[k], ref.f[k]), k
    if cu0 > 0:
        assert np.abs(ref.f["uss"]).max() > 0
