"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/_build/libwolfd2_oracle.so (building it with ``make`` when it is
missing) and exposes the restated reference routines on Fortran-layout numpy
arrays of shape (mnx+1, mny+1).  Used by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, never by the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwolfd2_oracle.so")
_lock = threading.Lock()
_lib = None

METRIC_NAMES = ("ran rbn rgn rac rbc rgc rau rbu rbv rgv dju djv djc djn "
                "xen yen xzn yzn xec yec xzc yzc xeu yeu xzv yzv xzu yzu xev yev").split()
FIELD_NAMES = "u v p t un vn pn tn us vs ts d dn".split()

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _Regions(C.Structure):
    _fields_ = [("mgri", C.c_int), ("mgrj", C.c_int), ("nReg", _ip),
                ("nRegBrd", _ip), ("nRegType", _ip), ("nMomBdTp", _ip),
                ("dBCVal", _dp), ("dPRporos", _dp), ("dPRporc1", _dp),
                ("dPRporc2", _dp), ("prof", C.POINTER(_dp))]


class _Metrics(C.Structure):
    _fields_ = [(n, _dp) for n in METRIC_NAMES]


class AtdParams(C.Structure):
    """w2o_atd_params: SmallScale's parameters (parse.f:144-178 defaults)."""
    _fields_ = [(n, C.c_int) for n in ("npsolver", "msorit", "lcartes")] + \
        [(n, C.c_double) for n in ("dlref", "uref", "tref", "tmax", "dka", "re", "pe", "sortol",
                                   "sorrel")] + \
        [("fp", C.c_double * 4)] + \
        [(n, C.c_double) for n in ("cu0", "tscoef", "hscoef", "temcoef", "bnumc", "rmax", "rlc")]

    @classmethod
    def make(cls, *, dka, re, pe, npsolver=1, msorit=2000, lcartes=1, dlref=1.0, uref=1.0,
             tref=300.0, tmax=330.0, sortol=1e-8, sorrel=1.0, fp=(500.0, 500.0, 0.0, 500.0),
             cu0=0.0, tscoef=1.0, hscoef=1.0, temcoef=1.0, bnumc=200.0, rmax=0.95, rlc=5.0):
        return cls(npsolver, msorit, lcartes, dlref, uref, tref, tmax, dka, re, pe, sortol, sorrel,
                   (C.c_double * 4)(*fp), cu0, tscoef, hscoef, temcoef, bnumc, rmax, rlc)


class _Thermal(C.Structure):
    _fields_ = [("nTRgType", _ip), ("nTemBdTp", _ip), ("dTRgVal", _dp), ("dHGSTval", _dp)]


_fp = C.POINTER(C.c_float)


class _Metrics32(C.Structure):
    _fields_ = [(n, _fp) for n in METRIC_NAMES]


class _Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in "dk re fr qtol sortol sorrel fpu fpv".split()] + \
               [(n, C.c_int) for n in "mqiter npsolver msorit nfiltu nfiltv lcartes".split()]


class _Fields(C.Structure):
    _fields_ = [(n, _dp) for n in FIELD_NAMES]


class _ThermalParams(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nthermen", "neqstate", "nmeiter")] + \
               [(n, C.c_double) for n in ("dmeittol", "pe", "uref", "densref", "tmax", "tref", "rconst")] + \
               [("nfiltt", C.c_int), ("fpt", C.c_double)]


def build(force: bool = False) -> str:
    """Compile the oracle library (gcc, no FMA contraction)."""
    srcs = ("wolfd2_oracle.c", "wolfd2_oracle.h", "momentum_impl.h")
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(os.path.join(HERE, f)) for f in srcs):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB_PATH)
            L.w2o_create.restype = C.c_void_p
            L.w2o_create.argtypes = [C.c_int, C.c_int]
            L.w2o_destroy.argtypes = [C.c_void_p]
            L.w2o_grid.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, C.POINTER(_Metrics)]
            L.w2o_naux_momentum.restype = C.c_int
            L.w2o_naux_momentum.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int,
                                            C.POINTER(_Regions), C.c_double, C.c_double,
                                            C.c_double, C.c_double, C.POINTER(_Metrics),
                                            _dp, _dp, _dp, _dp, _dp, _dp]
            L.w2o_naux_momentum_f32.restype = C.c_int
            L.w2o_naux_momentum_f32.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int,
                                                C.POINTER(_Regions), C.c_double, C.c_double,
                                                C.c_double, C.c_double, C.POINTER(_Metrics32),
                                                _fp, _fp, _fp, _fp, _fp, _fp]
            L.w2o_ppe.restype = C.c_int
            L.w2o_ppe.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions), C.c_int,
                                  C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                  C.POINTER(_Metrics), _dp, _dp, _dp]
            L.w2o_project.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions),
                                      C.c_double, C.POINTER(_Metrics), _dp, _dp, _dp]
            for nm in ("w2o_vel_bound_cond", "w2o_vel_outflow_bcs"):
                getattr(L, nm).argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions), _dp, _dp]
            L.w2o_pres_bound_cond.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions), _dp]
            L.w2o_filter.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(_Regions),
                                     C.c_double, _dp]
            L.w2o_diff_max_norm.restype = C.c_double
            L.w2o_diff_max_norm.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp]
            L.w2o_dmax_norm.restype = C.c_double
            L.w2o_dmax_norm.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp]
            L.w2o_alt_trid_lu.argtypes = [C.c_int, _dp, _dp]
            L.w2o_temp_bound_cond.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions),
                                              C.POINTER(_Thermal), _dp]
            L.w2o_therm_energy.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions),
                                           C.POINTER(_Thermal), C.c_double, C.c_double,
                                           C.POINTER(_Metrics), _dp, _dp, _dp, _dp, _dp, _dp]
            L.w2o_eq_state.argtypes = [C.c_void_p, C.c_int, C.c_int] + [C.c_double] * 5 + [_dp, _dp, _dp]
            L.w2o_atd_create.argtypes = [C.c_int, C.c_int]
            L.w2o_atd_create.restype = C.c_void_p
            L.w2o_atd_destroy.argtypes = [C.c_void_p]
            L.w2o_sml_scl_bc.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions),
                                         C.POINTER(_Thermal), _dp, _dp, _dp, _dp]
            L.w2o_small_scale.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                          C.POINTER(_Regions), C.POINTER(_Thermal),
                                          C.POINTER(AtdParams), C.POINTER(_Metrics)] + [_dp] * 7
            L.w2o_small_scale.restype = C.c_int
            L.w2o_step_atd.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions),
                                       C.POINTER(_Thermal), C.c_void_p, C.c_void_p,
                                       C.POINTER(_Metrics), C.c_void_p, C.c_void_p,
                                       C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]
            L.w2o_step_atd.restype = C.c_int
            L.w2o_filter_t.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions),
                                       C.POINTER(_Thermal), C.c_double, _dp]
            L.w2o_cold_start.restype = C.c_int
            L.w2o_cold_start.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions),
                                         C.POINTER(_Params), C.POINTER(_Metrics), C.POINTER(_Fields)]
            L.w2o_step_thermal.restype = C.c_int
            L.w2o_step_thermal.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions),
                                           C.POINTER(_Thermal), C.POINTER(_ThermalParams),
                                           C.POINTER(_Params), C.POINTER(_Metrics), C.POINTER(_Fields),
                                           _ip, _ip, _dp]
            L.w2o_step.restype = C.c_int
            L.w2o_step.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(_Regions),
                                   C.POINTER(_Params), C.POINTER(_Metrics), C.POINTER(_Fields),
                                   _ip, _ip, _dp]
            _lib = L
    return _lib


def _ptr(a: np.ndarray, ct=C.c_double):
    assert a.flags["F_CONTIGUOUS"] or a.ndim == 1, "oracle arrays must be Fortran-ordered"
    return a.ctypes.data_as(C.POINTER(ct))


def alt_trid_lu(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """AltTridLU on copies; a has shape (3, n) (Fortran a(3,n))."""
    a = np.asfortranarray(a, np.float64).copy(order="F")
    b = np.ascontiguousarray(b, np.float64).copy()
    lib().w2o_alt_trid_lu(int(b.size), _ptr(a), b.ctypes.data_as(_dp))
    return b


class Oracle:
    """One oracle context: persistent work arrays for a (0:mnx, 0:mny) box."""

    def __init__(self, mnx: int, mny: int):
        self.mnx, self.mny = mnx, mny
        self.L = lib()
        self.h = C.c_void_p(self.L.w2o_create(mnx, mny))
        self._keep = []

    def __del__(self):
        try:
            if self.h:
                self.L.w2o_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def field(self) -> np.ndarray:
        return np.zeros((self.mnx + 1, self.mny + 1), np.float64, order="F")

    # -- setup --------------------------------------------------------------
    def grid(self, nx: int, ny: int, x_nodes: np.ndarray, y_nodes: np.ndarray) -> Dict[str, np.ndarray]:
        """grid.f Grid minus file reading; returns the 30 metric arrays."""
        gx, gy = self.field(), self.field()
        gx[1:nx + 1, 1:ny + 1] = x_nodes
        gy[1:nx + 1, 1:ny + 1] = y_nodes
        met = {n: self.field() for n in METRIC_NAMES}
        ms = _Metrics(*[_ptr(met[n]) for n in METRIC_NAMES])
        self.L.w2o_grid(self.h, nx, ny, _ptr(gx), _ptr(gy), C.byref(ms))
        met["gx"], met["gy"] = gx, gy
        return met

    @staticmethod
    def regions_struct(regs) -> _Regions:
        arrs = [np.asfortranarray(getattr(regs, n)) for n in
                ("nReg", "nRegBrd", "nRegType", "nMomBdTp")]
        darrs = [np.asfortranarray(getattr(regs, n)) for n in
                 ("dBCVal", "dPRporos", "dPRporc1", "dPRporc2")]
        mgri, mgrj = regs.nRegBrd.shape[0], regs.nRegBrd.shape[1]
        profs = getattr(regs, "profiles", None) or {}
        table, keep = None, []
        if profs:
            table = (_dp * (mgri * mgrj * 4 * 2))()
            for (ir, jr, face, var), vals in profs.items():
                a = np.ascontiguousarray(vals, np.float64)
                keep.append(a)
                table[((ir - 1) + (jr - 1) * mgri + (face - 1) * mgri * mgrj) * 2 + (var - 1)] = \
                    a.ctypes.data_as(_dp)
        s = _Regions(mgri, mgrj, *[_ptr(a, C.c_int) for a in arrs], *[_ptr(a) for a in darrs],
                     C.cast(table, C.POINTER(_dp)) if table is not None else None)
        s._keep = (arrs, darrs, table, keep)
        return s

    @staticmethod
    def metrics_struct(met: Dict[str, np.ndarray]) -> _Metrics:
        return _Metrics(*[_ptr(met[n]) for n in METRIC_NAMES])

    @staticmethod
    def params_struct(p) -> _Params:
        return _Params(p.dk, p.re, p.fr, p.qtol, p.sortol, p.sorrel, p.fpu, p.fpv,
                       p.mqiter, p.npsolver, p.msorit, p.nfiltu, p.nfiltv, p.lcartes)

    # -- routines -----------------------------------------------------------
    def naux_momentum(self, nx, ny, regs, prm, met, d, dn, un, vn, us, vs) -> int:
        rs = self.regions_struct(regs)
        return self.L.w2o_naux_momentum(self.h, nx, ny, prm.mqiter, C.byref(rs), prm.dk,
                                        prm.re, prm.fr, prm.qtol,
                                        C.byref(self.metrics_struct(met)),
                                        _ptr(d), _ptr(dn), _ptr(un), _ptr(vn), _ptr(us), _ptr(vs))

    def field32(self) -> np.ndarray:
        return np.zeros((self.mnx + 1, self.mny + 1), np.float32, order="F")

    @staticmethod
    def metrics32(met: Dict[str, np.ndarray]) -> Dict[str, np.ndarray]:
        """The metric arrays rounded to single precision."""
        return {n: np.asfortranarray(met[n].astype(np.float32)) for n in METRIC_NAMES}

    def naux_momentum_f32(self, nx, ny, regs, prm, met32, d, dn, un, vn, us, vs) -> int:
        """nAuxMomentum in IEEE single on float32 Fortran-ordered arrays."""
        rs = self.regions_struct(regs)
        ms = _Metrics32(*[_ptr(met32[n], C.c_float) for n in METRIC_NAMES])
        f = [_ptr(a, C.c_float) for a in (d, dn, un, vn, us, vs)]
        for a in (d, dn, un, vn, us, vs):
            assert a.dtype == np.float32
        return self.L.w2o_naux_momentum_f32(self.h, nx, ny, prm.mqiter, C.byref(rs), prm.dk,
                                            prm.re, prm.fr, prm.qtol, C.byref(ms), *f)

    def ppe(self, nx, ny, regs, prm, met, u, v, p, npsolver=None, msorit=None) -> int:
        rs = self.regions_struct(regs)
        return self.L.w2o_ppe(self.h, nx, ny, C.byref(rs), prm.lcartes,
                              prm.npsolver if npsolver is None else npsolver,
                              prm.msorit if msorit is None else msorit,
                              prm.dk, prm.sortol, prm.sorrel,
                              C.byref(self.metrics_struct(met)), _ptr(u), _ptr(v), _ptr(p))

    def project(self, nx, ny, regs, dk, met, p, u, v) -> None:
        rs = self.regions_struct(regs)
        self.L.w2o_project(self.h, nx, ny, C.byref(rs), dk, C.byref(self.metrics_struct(met)),
                           _ptr(p), _ptr(u), _ptr(v))

    def vel_bound_cond(self, nx, ny, regs, u, v) -> None:
        rs = self.regions_struct(regs)
        self.L.w2o_vel_bound_cond(self.h, nx, ny, C.byref(rs), _ptr(u), _ptr(v))

    def vel_outflow_bcs(self, nx, ny, regs, u, v) -> None:
        rs = self.regions_struct(regs)
        self.L.w2o_vel_outflow_bcs(self.h, nx, ny, C.byref(rs), _ptr(u), _ptr(v))

    def pres_bound_cond(self, nx, ny, regs, p) -> None:
        rs = self.regions_struct(regs)
        self.L.w2o_pres_bound_cond(self.h, nx, ny, C.byref(rs), _ptr(p))

    def filter(self, nx, ny, ncomp, regs, fp, q) -> None:
        rs = self.regions_struct(regs)
        self.L.w2o_filter(self.h, nx, ny, ncomp, C.byref(rs), fp, _ptr(q))

    @staticmethod
    def thermal_struct(th) -> _Thermal:
        """th: an object with nTRgType (mgri, mgrj), nTemBdTp (mgri, mgrj, 4),
        dTRgVal and dHGSTval (mgri, mgrj), Fortran-ordered."""
        ia = [np.asfortranarray(getattr(th, n), np.int32) for n in ("nTRgType", "nTemBdTp")]
        da = [np.asfortranarray(getattr(th, n), np.float64) for n in ("dTRgVal", "dHGSTval")]
        s = _Thermal(*[_ptr(a, C.c_int) for a in ia], *[_ptr(a) for a in da])
        s._keep = (ia, da)
        return s

    def temp_bound_cond(self, nx, ny, regs, th, t) -> None:
        rs, ts = self.regions_struct(regs), self.thermal_struct(th)
        self.L.w2o_temp_bound_cond(self.h, nx, ny, C.byref(rs), C.byref(ts), _ptr(t))

    def therm_energy(self, nx, ny, regs, th, dk, pe, met, un, vn, u, v, tn, t) -> None:
        rs, ts = self.regions_struct(regs), self.thermal_struct(th)
        self.L.w2o_therm_energy(self.h, nx, ny, C.byref(rs), C.byref(ts), dk, pe,
                                C.byref(self.metrics_struct(met)), _ptr(un), _ptr(vn), _ptr(u),
                                _ptr(v), _ptr(tn), _ptr(t))

    def sml_scl_bc(self, nx, ny, regs, th, u, v, p, t) -> None:
        rs, ts = self.regions_struct(regs), self.thermal_struct(th)
        self.L.w2o_sml_scl_bc(self.h, nx, ny, C.byref(rs), C.byref(ts), _ptr(u), _ptr(v), _ptr(p),
                              _ptr(t))

    def filter_t(self, nx, ny, regs, th, fp, q) -> None:
        rs, ts = self.regions_struct(regs), self.thermal_struct(th)
        self.L.w2o_filter_t(self.h, nx, ny, C.byref(rs), C.byref(ts), fp, _ptr(q))

    def eq_state(self, nx, ny, uref, densref, tmax, tref, rconst, p, t, den) -> None:
        self.L.w2o_eq_state(self.h, nx, ny, uref, densref, tmax, tref, rconst, _ptr(p), _ptr(t), _ptr(den))

    def diff_max_norm(self, nx, ny, un, u) -> float:
        return self.L.w2o_diff_max_norm(self.h, nx, ny, _ptr(un), _ptr(u))

    def dmax_norm(self, nx, ny, u) -> float:
        return self.L.w2o_dmax_norm(self.h, nx, ny, _ptr(u))


class OracleRun:
    """A whole case advanced by the oracle's time loop (main.f:690-972)."""

    def __init__(self, case, fields: Optional[Dict[str, np.ndarray]] = None, cold_start: bool = True):
        self.case = case
        self.nx, self.ny = case.nx, case.ny
        self.o = Oracle(case.nx + 1, case.ny + 1)
        self.met = self.o.grid(case.nx, case.ny, case.x, case.y)
        self.f = {n: self.o.field() for n in FIELD_NAMES}
        if fields:
            for k, v in fields.items():
                self.f[k][...] = v
        self._rs = Oracle.regions_struct(case.regions)
        self._ms = Oracle.metrics_struct(self.met)
        self._ps = Oracle.params_struct(case.params)
        self._fs = _Fields(*[_ptr(self.f[n]) for n in FIELD_NAMES])
        self._th = self._tp = None
        if getattr(case, "thermal", None) is not None and getattr(case, "tparams", None) is not None:
            self._th = Oracle.thermal_struct(case.thermal)
            tp = case.tparams
            self._tp = _ThermalParams(tp.nthermen, tp.neqstate, tp.nmeiter, tp.dmeittol, tp.pe, tp.uref,
                                      tp.densref, tp.tmax, tp.tref, tp.rconst, tp.nfiltt, tp.fpt)
        self.history = []
        self.cold_nconv = None
        if cold_start:
            self.cold_nconv = self.o.L.w2o_cold_start(self.o.h, self.nx, self.ny, C.byref(self._rs),
                                                      C.byref(self._ps), C.byref(self._ms),
                                                      C.byref(self._fs))
        self.atd = None
        a = getattr(case, "atd", None)
        if a is not None:
            # main.f:645-664: the small scales seeded after the cold start
            from wolfd2_gb300.deck import Thermal
            th = case.thermal if case.thermal is not None else Thermal.empty()
            self._th_atd = Oracle.thermal_struct(th)
            p = case.params
            self._ap = AtdParams.make(dka=p.dk, re=p.re, pe=a.pe, npsolver=a.npsolver, msorit=a.msorit,
                                      lcartes=p.lcartes, dlref=a.dlref, uref=a.uref, tref=a.tref,
                                      tmax=a.tmax, sortol=a.sortol, sorrel=a.sorrel,
                                      fp=(a.fpu, a.fpv, 0.0, a.fpt), cu0=a.cu0, tscoef=a.tscoef,
                                      hscoef=a.hscoef, temcoef=a.temcoef, bnumc=a.bnumc,
                                      rmax=a.rmax, rlc=a.rlc)
            self.atd = SmallScale(self.o, self.nx, self.ny, case.regions, th, self.met, self._ap)
            for k in ("uss", "vss", "pss", "tss", "usn", "vsn", "tsn"):
                self.f[k] = self.o.field()
            f = self.f
            self.atd_nsor = [self.atd(0, f["u"], f["v"], f["t"], f["uss"], f["vss"], f["pss"], f["tss"])]
            self._run = _AtdRun(self.atd.s, C.pointer(self._ap),
                                *[_ptr(f[k]) for k in ("uss", "vss", "pss", "tss", "usn", "vsn", "tsn")])

    def step(self, n: int = 1):
        nql, nsor = C.c_int(), C.c_int()
        dif = (C.c_double * 4)()
        for _ in range(n):
            if self.atd is not None:
                tp = C.byref(self._tp) if self._tp is not None else None
                rc = self.o.L.w2o_step_atd(self.o.h, self.nx, self.ny, C.byref(self._rs),
                                           C.byref(self._th_atd), tp, C.byref(self._ps),
                                           C.byref(self._ms), C.byref(self._fs), C.byref(self._run),
                                           C.byref(nql), C.byref(nsor), dif)
            elif self._th is not None:
                rc = self.o.L.w2o_step_thermal(self.o.h, self.nx, self.ny, C.byref(self._rs),
                                               C.byref(self._th), C.byref(self._tp), C.byref(self._ps),
                                               C.byref(self._ms), C.byref(self._fs), C.byref(nql),
                                               C.byref(nsor), dif)
            else:
                rc = self.o.L.w2o_step(self.o.h, self.nx, self.ny, C.byref(self._rs), C.byref(self._ps),
                                       C.byref(self._ms), C.byref(self._fs), C.byref(nql),
                                       C.byref(nsor), dif)
            self.history.append((nql.value, nsor.value, tuple(dif)))
            if rc:
                raise FloatingPointError("Solution diverged. Please reduce CFL number.")
        return self.history[-1] if self.history else None


def threads() -> int:
    """Host threads the oracle library runs on (1: the restatement is serial,
    like the reference)."""
    return 1


class _AtdRun(C.Structure):
    _fields_ = [("state", C.c_void_p), ("ap", C.POINTER(AtdParams))] + \
        [(k, _dp) for k in ("uss", "vss", "pss", "tss", "usn", "vsn", "tsn")]


class SmallScale:
    """small_scale.f's SmallScale with its saved state (the map iterates,
    cell areas and work arrays) held by this object instead of static
    storage; one object per run."""

    def __init__(self, o: "Oracle", nx: int, ny: int, regs, th, met, ap: AtdParams):
        self.o, self.nx, self.ny = o, nx, ny
        self.s = o.L.w2o_atd_create(o.mnx, o.mny)
        self._rs, self._ts = Oracle.regions_struct(regs), Oracle.thermal_struct(th)
        self._ms = Oracle.metrics_struct(met)
        self.ap = ap

    def __call__(self, initflg, u1, v1, t1, uss, vss, pss, tss) -> int:
        return self.o.L.w2o_small_scale(self.o.h, self.s, self.nx, self.ny, initflg,
                                        C.byref(self._rs), C.byref(self._ts), C.byref(self.ap),
                                        C.byref(self._ms), _ptr(u1), _ptr(v1), _ptr(t1), _ptr(uss),
                                        _ptr(vss), _ptr(pss), _ptr(tss))

    def __del__(self):
        if getattr(self, "s", None):
            self.o.L.w2o_atd_destroy(self.s)
            self.s = None
