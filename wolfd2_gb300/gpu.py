"""ctypes binding of the C-ABI in include/wolfd2_gpu.h.

The class :class:`Solver` mirrors the reference's hot-path subroutines by
name and argument meaning -- ``nAuxMomentum``, ``Ppe``, ``Project``,
``VelBoundCond``, ``PresBoundCond``, ``VelOutflowBCs``, ``DiffMaxNorm``,
``Filter`` -- operating on Fortran-layout numpy arrays of shape
(mnx+1, mny+1) exactly like the Fortran driver's static arrays, plus the
device-resident time loop (``load_fields`` / ``cold_start`` / ``step`` /
``store_fields``).

There is no CPU fallback: if the CUDA library is missing or no GPU is
visible, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import build as _build
from .deck import Case, Regions, RunParams

W2_OK = 0
ERRORS = {1: "bad argument", 2: "CUDA error", 3: "device wait timed out",
          4: "solution diverged", 5: "invalid boundary flag",
          6: "unsupported configuration", 7: "chain fallback",
          8: "larger than the allocation-free scratch"}
NOALLOC_MAX_POINTS = 1200000
PREC_FP64, PREC_MIXED = 0, 1
K_MOMENTUM, K_PPE, K_POST, K_BC, K_COPY, K_THERM = range(6)
KERNEL_NAMES = {K_MOMENTUM: "k_naux", K_PPE: "k_ppe", K_POST: "k_step_post",
                K_BC: "k_bc", K_COPY: "k_copy3", K_THERM: "k_therm"}


class ThermalC(C.Structure):
    """w2_thermal of include/wolfd2_gpu.h."""
    _fields_ = [(n, C.c_int) for n in ("nthermen", "neqstate", "nmeiter")] + \
               [(n, C.c_double) for n in ("dmeittol", "pe", "uref", "densref", "tmax", "tref", "rconst")] + \
               [("nfiltt", C.c_int), ("fpt", C.c_double)]

# metric order of the C-ABI = argument order of grid.f:Grid
METRIC_ORDER = ("rau rbu rbv rgv ran rbn rgn rac rbc rgc dju djv djc djn xen yen xzn yzn "
                "xec yec xzc yzc xeu yeu xzv yzv xzu yzu xev yev").split()

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class W2Error(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"wolfd2gpu error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in "dk re fr qtol sortol sorrel fpu fpv".split()] + \
               [(n, C.c_int) for n in "mqiter npsolver msorit nfiltu nfiltv lcartes precision refine_sweeps".split()] + \
               [("refine_tol", C.c_double)]

    @staticmethod
    def of(p: RunParams, precision: int = PREC_FP64, refine_sweeps: int = 0,
           refine_tol: float = 0.0) -> "Params":
        return Params(p.dk, p.re, p.fr, p.qtol, p.sortol, p.sorrel, p.fpu, p.fpv,
                      p.mqiter, p.npsolver, p.msorit, p.nfiltu, p.nfiltv, p.lcartes,
                      precision, refine_sweeps, refine_tol)


class StepStat(C.Structure):
    _fields_ = [("nQLiter", C.c_int), ("nSorConv", C.c_int), ("dif", C.c_double * 4),
                ("divmax", C.c_double), ("divmax_int", C.c_double)]


_lib = None


def library_path() -> str:
    return _build.LIB


def lib():
    """Load libwolfd2gpu.so (building it in-tree when sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if _build.needs_build():
        _build.build_library()
    if not os.path.exists(_build.LIB):
        raise RuntimeError(f"CUDA library missing: {_build.LIB}")
    L = C.CDLL(_build.LIB)
    vp = C.c_void_p
    L.wolfd2gpu_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_int, _ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp]
    L.wolfd2gpu_destroy.argtypes = [vp]
    L.wolfd2gpu_set_metrics.argtypes = [vp, C.POINTER(_dp)]
    L.wolfd2gpu_grid_metric.argtypes = [vp, _dp, _dp, C.POINTER(_dp)]
    L.wolfd2gpu_naux_momentum.argtypes = [vp, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp,
                                          _dp, _dp, _dp, _dp, _ip]
    L.wolfd2gpu_ppe.argtypes = [vp, _ip, _ip, _ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp]
    L.wolfd2gpu_project.argtypes = [vp, _ip, _ip, _dp, _dp, _dp, _dp]
    L.wolfd2gpu_vel_bound_cond.argtypes = [vp, _ip, _ip, _dp, _dp]
    L.wolfd2gpu_pres_bound_cond.argtypes = [vp, _ip, _ip, _dp]
    L.wolfd2gpu_vel_outflow_bcs.argtypes = [vp, _ip, _ip, _dp, _dp]
    L.wolfd2gpu_diff_max_norm.argtypes = [vp, _ip, _ip, _dp, _dp, _dp]
    L.wolfd2gpu_filter.argtypes = [vp, _ip, _ip, _ip, _dp, _dp]
    L.wolfd2gpu_temp_bound_cond.argtypes = [vp, _ip, _ip, _ip, _ip, _dp, _dp]
    L.wolfd2gpu_therm_energy.argtypes = [vp, _ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp] + [_dp] * 6
    L.wolfd2gpu_eq_state.argtypes = [vp, _ip, _ip] + [_dp] * 8
    # ctx; nx ny initflg nthermen lCartesGrid nTRgType nTemBdTp nPpeSolver msorit;
    # dlref uref tref tmax dka re pe sortol sorrel; fp; cu0 TsCoef HsCoef TemCoef
    # bnumc rmax rlc; dTRgVal; u1 v1 t1 uss vss pss tss; nSorConv
    L.wolfd2gpu_small_scale.argtypes = [vp] + [_ip] * 9 + [_dp] * 9 + [_dp] + [_dp] * 7 + [_dp] + \
        [_dp] * 7 + [_ip]
    L.wolfd2gpu_filter_t.argtypes = [vp, _ip, _ip, _ip, _dp, _dp]
    L.wolfd2gpu_set_thermal.argtypes = [vp, C.POINTER(ThermalC), _ip, _ip, _dp, _dp]
    L.wolfd2gpu_load_thermal.argtypes = [vp, _dp, _dp]
    L.wolfd2gpu_store_thermal.argtypes = [vp, _dp, _dp]
    L.wolfd2gpu_snapshot.argtypes = [vp, _dp, _dp, _dp, _dp, _dp]
    L.wolfd2gpu_snapshot_wait.argtypes = [vp]
    L.wolfd2gpu_selftest_wait.argtypes = [vp]
    L.wolfd2gpu_load_fields.argtypes = [vp, _dp, _dp, _dp]
    L.wolfd2gpu_store_fields.argtypes = [vp, _dp, _dp, _dp]
    L.wolfd2gpu_cold_start.argtypes = [vp, C.POINTER(Params), _ip]
    L.wolfd2gpu_step.argtypes = [vp, C.POINTER(Params), C.c_int, C.POINTER(StepStat)]
    L.wolfd2gpu_sync.argtypes = [vp]
    L.wolfd2gpu_last_error.argtypes = [vp]
    L.wolfd2gpu_last_error.restype = C.c_char_p
    L.wolfd2gpu_tune.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
    L.wolfd2gpu_tune_mixed.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    L.wolfd2gpu_set_precision.argtypes = [vp, C.c_int, C.c_int]
    L.wolfd2gpu_set_tma.argtypes = [vp, C.c_int]
    L.wolfd2gpu_set_face_profile.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, C.c_int]
    L.wolfd2gpu_device_fields.argtypes = [vp, C.POINTER(_dp), C.POINTER(_dp), C.POINTER(_dp), _ip]
    L.wolfd2gpu_launch_count.argtypes = [vp]
    L.wolfd2gpu_launch_count.restype = C.c_longlong
    L.wolfd2gpu_stream.argtypes = [vp]
    L.wolfd2gpu_stream.restype = C.c_void_p
    L.wolfd2gpu_profile.argtypes = [vp, C.c_int]
    L.wolfd2gpu_set_graph.argtypes = [vp, C.c_int]
    L.wolfd2gpu_step_counts.argtypes = [vp, C.POINTER(Params), C.c_int, _ip, C.POINTER(StepStat)]
    L.wolfd2gpu_adjoint.argtypes = [vp, C.POINTER(Params), C.c_int, C.c_int, C.c_double, _dp, _dp, _dp,
                                    _dp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.c_int, _ip]
    L.wolfd2gpu_chain_stats.argtypes = [vp, _ip, _ip]
    L.wolfd2gpu_ppe_rbsor_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                              C.c_double, C.c_double, C.c_double] + [vp] * 9 + [_ip, vp]
    L.wolfd2gpu_profile_read.argtypes = [vp, C.c_int, _dp, C.POINTER(C.c_longlong)]
    L.wolfd2gpu_ens_create.argtypes = [C.POINTER(vp), C.POINTER(vp), C.c_int, C.c_int, C.c_int]
    L.wolfd2gpu_ens_step.argtypes = [vp, C.POINTER(Params), C.c_int, C.POINTER(StepStat)]
    L.wolfd2gpu_ens_graph.argtypes = [vp, C.c_int]
    L.wolfd2gpu_ens_info.argtypes = [vp, _ip, _ip, _dp, C.POINTER(C.c_longlong)]
    L.wolfd2gpu_ens_error.argtypes = [vp]
    L.wolfd2gpu_ens_error.restype = C.c_char_p
    L.wolfd2gpu_ens_destroy.argtypes = [vp]
    L.wolfd2gpu_ens_profile.argtypes = [vp, C.c_int]
    L.wolfd2gpu_ens_profile_read.argtypes = [vp, C.c_int, _dp, C.POINTER(C.c_longlong)]
    _lib = L
    return L


def _p(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags["F_CONTIGUOUS"]:
        raise TypeError("expected a Fortran-ordered float64 array")
    return a.ctypes.data_as(_dp)


def _i(v: int):
    return C.byref(C.c_int(int(v)))


def _d(v: float):
    return C.byref(C.c_double(float(v)))


def ppe_rbsor_noalloc(nx, ny, ld, msorit, dk, sortol, sorrel, rau, rgv, xeu, yeu, xzv, yzv,
                      u, v, p, stream=0, lcartes=1, npsolver=5) -> int:
    """Allocation-free red/black Ppe on device arrays (integer device
    addresses in the reference layout with leading dimension ld); returns
    nSorConv.  See wolfd2gpu_ppe_rbsor_noalloc in include/wolfd2_gpu.h."""
    L = lib()
    out = C.c_int()
    rc = L.wolfd2gpu_ppe_rbsor_noalloc(nx, ny, ld, lcartes, npsolver, msorit, dk, sortol, sorrel,
                                       rau, rgv, xeu, yeu, xzv, yzv, u, v, p, C.byref(out),
                                       stream or None)
    if rc != W2_OK:
        raise W2Error(rc, "wolfd2gpu_ppe_rbsor_noalloc failed")
    return out.value


class Solver:
    """One device context for an nx x ny grid with the given region tables."""

    def __init__(self, nx: int, ny: int, regions: Regions, mnx: Optional[int] = None,
                 mny: Optional[int] = None):
        self.L = lib()
        self.nx, self.ny = nx, ny
        self.mnx = nx + 1 if mnx is None else mnx
        self.mny = ny + 1 if mny is None else mny
        self.regions = regions
        self._keep = [np.ascontiguousarray(regions.nReg, np.int32)] + \
            [np.asfortranarray(getattr(regions, n)) for n in ("nRegBrd", "nRegType", "nMomBdTp")] + \
            [np.asfortranarray(getattr(regions, n)) for n in ("dBCVal", "dPRporos", "dPRporc1", "dPRporc2")]
        k = self._keep
        h = C.c_void_p()
        rc = self.L.wolfd2gpu_create(C.byref(h), self.mnx, self.mny, regions.nRegBrd.shape[0],
                                     regions.nRegBrd.shape[1], nx, ny,
                                     k[0].ctypes.data_as(_ip), k[1].ctypes.data_as(_ip),
                                     k[2].ctypes.data_as(_ip), k[3].ctypes.data_as(_ip),
                                     _p(k[4]), _p(k[5]), _p(k[6]), _p(k[7]))
        if rc != W2_OK:
            raise W2Error(rc, "wolfd2gpu_create failed")
        self.h = h
        self.refine_sweeps = 0  # mixed: FP32 sweeps per refinement pass (0 = library default)

    @classmethod
    def for_case(cls, case: Case, mnx: Optional[int] = None, mny: Optional[int] = None,
                 tuned: bool = True, precision: str = "mixed") -> "Solver":
        """Context for a case with its grid metrics; with `tuned`, the kernel
        shapes the autotuner committed for this grid shape (tuned.json)."""
        s = cls(case.nx, case.ny, case.regions, mnx, mny)
        s.grid_metric(case.x, case.y)
        for (ir, jr, face, var), vals in getattr(case.regions, "profiles", {}).items():
            s.set_face_profile(ir, jr, face, var, vals)
        if getattr(case, "tparams", None) is not None and getattr(case, "thermal", None) is not None:
            s.set_thermal(case.tparams, case.thermal)
        if tuned:
            from . import autotune
            autotune.apply(s, autotune.lookup(case.nx, case.ny, precision))
        return s

    def close(self):
        if getattr(self, "h", None):
            self.L.wolfd2gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != W2_OK:
            msg = self.L.wolfd2gpu_last_error(self.h).decode(errors="replace")
            raise W2Error(rc, msg)

    def field(self) -> np.ndarray:
        return np.zeros((self.mnx + 1, self.mny + 1), np.float64, order="F")

    # ---- set-up ------------------------------------------------------------
    def set_metrics(self, met: Dict[str, np.ndarray]) -> None:
        arr = (_dp * 30)(*[_p(met[n]) for n in METRIC_ORDER])
        self._check(self.L.wolfd2gpu_set_metrics(self.h, arr))

    def grid_metric(self, x_nodes: np.ndarray, y_nodes: np.ndarray,
                    want: bool = False) -> Optional[Dict[str, np.ndarray]]:
        gx, gy = self.field(), self.field()
        gx[1:self.nx + 1, 1:self.ny + 1] = x_nodes
        gy[1:self.nx + 1, 1:self.ny + 1] = y_nodes
        out = None
        outp = None
        if want:
            out = {n: self.field() for n in METRIC_ORDER}
            outp = (_dp * 30)(*[_p(out[n]) for n in METRIC_ORDER])
        self._check(self.L.wolfd2gpu_grid_metric(self.h, _p(gx), _p(gy), outp))
        return out

    def tune(self, seg: int = 0, warm: int = 0, threads: int = 0, blocks_per_sm: int = 0):
        self._check(self.L.wolfd2gpu_tune(self.h, seg, warm, threads, blocks_per_sm))

    def tune_mixed(self, sweeps_per_barrier: int = 0, threads: int = 0, mode: int = 0):
        """Mixed Poisson kernel shape: sweeps between grid barriers (4, 8),
        the block-size limit (0 keeps the current value), and the tile mode
        (0 auto, 1 several tiles per block, 2 the same on <= 16 blocks, 3 one
        tile per block with two blocks per SM)."""
        self._check(self.L.wolfd2gpu_tune_mixed(self.h, sweeps_per_barrier, threads, mode))

    def set_tma(self, enable: bool = True):
        """TMA staging of the mixed Poisson boxes in the several-tiles-per-
        block mode (default on; off: vector loads, same results)."""
        self._check(self.L.wolfd2gpu_set_tma(self.h, 1 if enable else 0))

    def set_face_profile(self, ireg: int, jreg: int, face: int, var: int, values=None):
        """Per-position inlet / moving-wall values on one region face (var 1 =
        u, 2 = v; values over j for west/east faces, over i for south/north);
        None restores the region constant."""
        if values is None:
            self._check(self.L.wolfd2gpu_set_face_profile(self.h, ireg, jreg, face, var, None, 0))
            return
        a = np.ascontiguousarray(values, np.float64)
        self._check(self.L.wolfd2gpu_set_face_profile(self.h, ireg, jreg, face, var,
                                                      a.ctypes.data_as(C.c_void_p), a.size))

    def set_precision(self, precision: int, refine_sweeps: int = 0):
        """Precision of the drop-in Ppe (PREC_FP64 or PREC_MIXED)."""
        self._check(self.L.wolfd2gpu_set_precision(self.h, precision, refine_sweeps))

    # ---- reference drop-ins ------------------------------------------------
    def nAuxMomentum(self, mqiter, dk, re, fr, qtol, d, dn, un, vn, us, vs) -> int:
        out = C.c_int()
        self._check(self.L.wolfd2gpu_naux_momentum(
            self.h, _i(self.nx), _i(self.ny), _i(mqiter), _d(dk), _d(re), _d(fr), _d(qtol),
            None if d is None else _p(d), None if dn is None else _p(dn),
            _p(un), _p(vn), _p(us), _p(vs), C.byref(out)))
        return out.value

    def Ppe(self, lCartesGrid, nPpeSolver, msorit, dk, sortol, sorrel, u, v, p) -> int:
        out = C.c_int()
        self._check(self.L.wolfd2gpu_ppe(
            self.h, _i(self.nx), _i(self.ny), _i(1 if lCartesGrid else 0), _i(nPpeSolver),
            _i(msorit), C.byref(out), _d(dk), _d(sortol), _d(sorrel), _p(u), _p(v), _p(p)))
        return out.value

    def Project(self, dk, p, u, v) -> None:
        self._check(self.L.wolfd2gpu_project(self.h, _i(self.nx), _i(self.ny), _d(dk), _p(p), _p(u), _p(v)))

    def VelBoundCond(self, u, v) -> None:
        self._check(self.L.wolfd2gpu_vel_bound_cond(self.h, _i(self.nx), _i(self.ny), _p(u), _p(v)))

    def PresBoundCond(self, p) -> None:
        self._check(self.L.wolfd2gpu_pres_bound_cond(self.h, _i(self.nx), _i(self.ny), _p(p)))

    def VelOutflowBCs(self, u, v) -> None:
        self._check(self.L.wolfd2gpu_vel_outflow_bcs(self.h, _i(self.nx), _i(self.ny), _p(u), _p(v)))

    def DiffMaxNorm(self, un, u) -> float:
        out = C.c_double()
        self._check(self.L.wolfd2gpu_diff_max_norm(self.h, _i(self.nx), _i(self.ny), _p(un), _p(u),
                                                   C.byref(out)))
        return out.value

    def Filter(self, ncomp, fp, qu) -> None:
        self._check(self.L.wolfd2gpu_filter(self.h, _i(self.nx), _i(self.ny), _i(ncomp), _d(fp), _p(qu)))

    @staticmethod
    def _ttab(a, dtype):
        a = np.asfortranarray(a, dtype)
        return a, a.ctypes.data_as(C.POINTER(C.c_int if dtype == np.int32 else C.c_double))

    def TempBoundCond(self, th, t) -> None:
        """th: deck.Thermal tables; t updated in place."""
        rt, prt = self._ttab(th.nTRgType, np.int32)
        bt, pbt = self._ttab(th.nTemBdTp, np.int32)
        tv, ptv = self._ttab(th.dTRgVal, np.float64)
        self._check(self.L.wolfd2gpu_temp_bound_cond(self.h, _i(self.nx), _i(self.ny), prt, pbt, ptv, _p(t)))

    def ThermEnergy(self, th, dk, pe, un, vn, u, v, tn, t) -> None:
        """ThermEnergy with deck.Thermal tables; t updated in place."""
        rt, prt = self._ttab(th.nTRgType, np.int32)
        bt, pbt = self._ttab(th.nTemBdTp, np.int32)
        tv, ptv = self._ttab(th.dTRgVal, np.float64)
        hg, phg = self._ttab(th.dHGSTval, np.float64)
        self._check(self.L.wolfd2gpu_therm_energy(
            self.h, _i(self.nx), _i(self.ny), prt, pbt, _d(dk), _d(pe), ptv, phg,
            _p(un), _p(vn), _p(u), _p(v), _p(tn), _p(t)))

    def FilterT(self, th, fp, t) -> None:
        """Filter of the temperature (utility.f, ncomp = _T_) in place."""
        rt, prt = self._ttab(th.nTRgType, np.int32)
        self._check(self.L.wolfd2gpu_filter_t(self.h, _i(self.nx), _i(self.ny), prt, _d(fp), _p(t)))

    def SmallScale(self, initflg, th, ap, u1, v1, t1, uss, vss, pss, tss, nthermen=1) -> int:
        """SmallScale (small_scale.f:31-49) on the device: the small-scale
        fields uss, vss, pss, tss (updated in place) from the large-scale u1,
        v1, t1.  th: deck.Thermal tables; ap: the routine's parameters
        (npsolver, msorit, lcartes, dlref, uref, tref, tmax, dka, re, pe,
        sortol, sorrel, fp[4], cu0, tscoef, hscoef, temcoef, bnumc, rmax,
        rlc).  The maps and cell areas persist in the context between calls,
        as the reference's SAVE keeps them.  Returns the Ppe's nSorConv."""
        rt, prt = self._ttab(th.nTRgType, np.int32)
        bt, pbt = self._ttab(th.nTemBdTp, np.int32)
        tv, ptv = self._ttab(th.dTRgVal, np.float64)
        fp = np.ascontiguousarray([float(x) for x in ap.fp], dtype=np.float64)
        out = C.c_int()
        self._check(self.L.wolfd2gpu_small_scale(
            self.h, _i(self.nx), _i(self.ny), _i(initflg), _i(nthermen), _i(ap.lcartes), prt, pbt,
            _i(ap.npsolver), _i(ap.msorit), _d(ap.dlref), _d(ap.uref), _d(ap.tref), _d(ap.tmax),
            _d(ap.dka), _d(ap.re), _d(ap.pe), _d(ap.sortol), _d(ap.sorrel),
            fp.ctypes.data_as(_dp), _d(ap.cu0), _d(ap.tscoef), _d(ap.hscoef), _d(ap.temcoef),
            _d(ap.bnumc), _d(ap.rmax), _d(ap.rlc), ptv, _p(u1), _p(v1), _p(t1), _p(uss), _p(vss),
            _p(pss), _p(tss), C.byref(out)))
        return out.value

    def EqState(self, uref, densref, tmax, tref, rconst, p, t, den) -> None:
        self._check(self.L.wolfd2gpu_eq_state(self.h, _i(self.nx), _i(self.ny), _d(uref), _d(densref),
                                              _d(tmax), _d(tref), _d(rconst), _p(p), _p(t), _p(den)))

    # ---- device-resident time loop ---------------------------------------
    def set_thermal(self, tparams=None, th=None) -> None:
        """Time loop with the energy equation (deck.ThermalParams and
        deck.Thermal tables); None returns to the plain loop."""
        if tparams is None:
            self._check(self.L.wolfd2gpu_set_thermal(self.h, None, None, None, None, None))
            return
        tp = tparams
        c = ThermalC(tp.nthermen, tp.neqstate, tp.nmeiter, tp.dmeittol, tp.pe, tp.uref, tp.densref,
                     tp.tmax, tp.tref, tp.rconst, tp.nfiltt, tp.fpt)
        rt, prt = self._ttab(th.nTRgType, np.int32)
        bt, pbt = self._ttab(th.nTemBdTp, np.int32)
        tv, ptv = self._ttab(th.dTRgVal, np.float64)
        hg, phg = self._ttab(th.dHGSTval, np.float64)
        self._check(self.L.wolfd2gpu_set_thermal(self.h, C.byref(c), prt, pbt, ptv, phg))

    def load_thermal(self, t, d=None) -> None:
        self._check(self.L.wolfd2gpu_load_thermal(self.h, _p(t), None if d is None else _p(d)))

    def store_thermal(self, out=None):
        """(t, d) to new host arrays, or t alone into `out` (a Fortran-ordered
        float64 array, for example a pinned buffer); returns (t, d)."""
        if out is not None:
            self._check(self.L.wolfd2gpu_store_thermal(self.h, _p(out), None))
            return out, None
        t = np.zeros((self.mnx + 1, self.mny + 1), order="F")
        d = np.zeros_like(t)
        self._check(self.L.wolfd2gpu_store_thermal(self.h, _p(t), _p(d)))
        return t, d

    def snapshot(self, out) -> None:
        """Queue a copy of the current level into the host arrays of `out`
        ((u, v, p) or (u, v, p, t, d), Fortran-ordered float64, page-locked
        for a copy that overlaps later steps) and return at once;
        snapshot_wait() blocks until they are filled."""
        arrs = list(out) + [None] * (5 - len(out))
        self._check(self.L.wolfd2gpu_snapshot(self.h, *[None if a is None else _p(a) for a in arrs]))

    def snapshot_wait(self) -> None:
        self._check(self.L.wolfd2gpu_snapshot_wait(self.h))

    def selftest_wait(self) -> int:
        """Status of a grid barrier one block never reaches (W2_E_TIMEOUT
        after the device-wait limit); the context stays usable."""
        return int(self.L.wolfd2gpu_selftest_wait(self.h))

    def load_fields(self, u, v, p) -> None:
        self._check(self.L.wolfd2gpu_load_fields(self.h, _p(u), _p(v), _p(p)))

    def store_fields(self, out=None):
        """Copy u, v, p to host arrays: new ones, or the three Fortran-ordered
        float64 arrays of `out` (for example pinned buffers)."""
        u, v, p = out if out is not None else (self.field(), self.field(), self.field())
        self._check(self.L.wolfd2gpu_store_fields(self.h, _p(u), _p(v), _p(p)))
        return u, v, p

    def cold_start(self, prm: RunParams, **kw) -> int:
        out = C.c_int()
        if kw.get("precision") == PREC_MIXED and not kw.get("refine_sweeps"):
            kw["refine_sweeps"] = self.refine_sweeps
        pr = Params.of(prm, **kw)
        self._check(self.L.wolfd2gpu_cold_start(self.h, C.byref(pr), C.byref(out)))
        return out.value

    def step(self, prm: RunParams, nsteps: int = 1, **kw) -> List[tuple]:
        if kw.get("precision") == PREC_MIXED and not kw.get("refine_sweeps"):
            kw["refine_sweeps"] = self.refine_sweeps
        pr = Params.of(prm, **kw)
        st = (StepStat * max(nsteps, 1))()
        self._check(self.L.wolfd2gpu_step(self.h, C.byref(pr), nsteps, st))
        return [(s.nQLiter, s.nSorConv, tuple(s.dif), s.divmax, s.divmax_int) for s in st[:nsteps]]

    def step_log(self, prm: RunParams, nsteps: int, path: str, k0: int = 0, dtime0: float = 0.0,
                 **kw) -> List[tuple]:
        """nsteps steps, then one JSON line per step appended to `path` with
        the fields of the reference's PrintDiff table (src/string.f:467-566):
        step k, dimensionless time, nQLiter, nSorConv and the max-norm
        differences of p, u, v (and t), plus the divergence check."""
        import json
        import math
        hist = self.step(prm, nsteps, **kw)
        with open(path, "a") as fh:
            for n, (nql, nsor, dif, divmax, divmax_int) in enumerate(hist, 1):
                rec = {"k": k0 + n, "time": dtime0 + n * prm.dk, "nQLiter": nql, "nSorConv": nsor,
                       "dif": [None if math.isnan(x) else x for x in dif], "divmax": divmax,
                       "divmax_interior": divmax_int}
                fh.write(json.dumps(rec) + "\n")
        return hist

    def step_counts(self, prm: RunParams, counts) -> List[tuple]:
        """Plain steps with each step's (Q-L iterations, SOR sweeps) fixed."""
        counts = np.ascontiguousarray(np.asarray(counts, dtype=np.int32).ravel())
        n = counts.size // 2
        pr = Params.of(prm)
        st = (StepStat * max(n, 1))()
        self._check(self.L.wolfd2gpu_step_counts(self.h, C.byref(pr), n, counts.ctypes.data_as(_ip), st))
        return [(s.nQLiter, s.nSorConv, tuple(s.dif), s.divmax, s.divmax_int) for s in st[:n]]

    def adjoint(self, prm: RunParams, nsteps: int, every: int = 20, weight: float = 1.0,
                profile=None, nprof: int = 0):
        """J = 0.5 * weight * sum(u^2 + v^2) over the momentum unknowns after
        nsteps plain steps from the loaded fields, and its gradient with the
        recorded iteration counts held fixed.  profile = (ireg, jreg, face,
        var) selects the face profile whose gradient is returned.  Returns
        (J, du, dv, dp, dprof, counts)."""
        gu, gv, gp = self.field(), self.field(), self.field()
        ir, jr, fc, vr = profile if profile else (0, 0, 0, 0)
        npf = nprof if profile else 0
        gprof = np.zeros(max(npf, 1))
        counts = np.zeros(2 * nsteps, dtype=np.int32)
        J = C.c_double()
        pr = Params.of(prm)
        self._check(self.L.wolfd2gpu_adjoint(self.h, C.byref(pr), nsteps, every, weight, C.byref(J), _p(gu),
                                             _p(gv), _p(gp), ir, jr, fc, vr, gprof.ctypes.data_as(_dp), npf,
                                             counts.ctypes.data_as(_ip)))
        return J.value, gu, gv, gp, gprof[:npf], counts.reshape(nsteps, 2)

    def sync(self) -> None:
        self._check(self.L.wolfd2gpu_sync(self.h))

    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return int(self.L.wolfd2gpu_stream(self.h) or 0)

    def profile(self, enable: bool = True) -> None:
        """Per-kernel CUDA-event timing (steps then launch directly, not
        from a captured graph)."""
        self._check(self.L.wolfd2gpu_profile(self.h, 1 if enable else 0))

    def graph(self, enable: bool = True) -> None:
        """Replay wolfd2gpu_step's launch sequences from captured CUDA graphs
        (the library default)."""
        self._check(self.L.wolfd2gpu_set_graph(self.h, 1 if enable else 0))

    def profile_read(self, kind: int):
        ms, n = C.c_double(), C.c_longlong()
        self._check(self.L.wolfd2gpu_profile_read(self.h, kind, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def chain_stats(self):
        """(most verification rounds used, sequential fallbacks) since the
        previous call."""
        r, f = C.c_int(), C.c_int()
        self._check(self.L.wolfd2gpu_chain_stats(self.h, C.byref(r), C.byref(f)))
        return r.value, f.value

    def launch_count(self) -> int:
        return int(self.L.wolfd2gpu_launch_count(self.h))

    def device_fields(self):
        u, v, p = _dp(), _dp(), _dp()
        ld = C.c_int()
        self._check(self.L.wolfd2gpu_device_fields(self.h, C.byref(u), C.byref(v), C.byref(p), C.byref(ld)))
        return (C.cast(u, C.c_void_p).value, C.cast(v, C.c_void_p).value,
                C.cast(p, C.c_void_p).value, ld.value)


class Ensemble:
    """Many independent cases advanced together, one launch per stage for
    all of them (wolfd2gpu_ens_*), by the mixed step or the plain FP64 step.
    Each case is an ordinary Solver, set up and loaded as usual;
    store_fields on a member reads that case's state.  The members must
    stay open while the ensemble is used."""

    def __init__(self, solvers: Sequence["Solver"], threads: int = 0, sweeps_per_barrier: int = 0,
                 graph: bool = True):
        self.L = lib()
        self.solvers = list(solvers)
        hs = (C.c_void_p * len(self.solvers))(*[s.h for s in self.solvers])
        h = C.c_void_p()
        rc = self.L.wolfd2gpu_ens_create(C.byref(h), hs, len(self.solvers), threads, sweeps_per_barrier)
        if rc:
            raise W2Error(rc, "ensemble creation failed (see stderr)")
        self.h = h
        self.L.wolfd2gpu_ens_graph(self.h, 1 if graph else 0)

    def _check(self, rc: int) -> None:
        if rc:
            raise W2Error(rc, self.L.wolfd2gpu_ens_error(self.h).decode())

    def step(self, params: Sequence[RunParams], nsteps: int = 1, refine_sweeps: int = 0,
             precision: int = PREC_MIXED) -> List[List[tuple]]:
        """nsteps steps of every case in `precision` (PREC_MIXED or
        PREC_FP64); returns per case the records (nQLiter, nSorConv, dif,
        divmax, divmax_int) of each step."""
        n = len(self.solvers)
        if len(params) != n:
            raise ValueError("one RunParams per case")
        pr = (Params * n)(*[Params.of(p, precision=precision, refine_sweeps=refine_sweeps) for p in params])
        st = (StepStat * max(n * nsteps, 1))()
        self._check(self.L.wolfd2gpu_ens_step(self.h, pr, nsteps, st))
        return [[(x.nQLiter, x.nSorConv, tuple(x.dif), x.divmax, x.divmax_int) for x in st[k * nsteps:(k + 1) * nsteps]]
                for k in range(n)]

    STAGES = ("ke_copy_mixed", "ke_naux32", "ke_bc", "ke_ppe_mixed", "ke_step_post")
    STAGES_FP64 = ("ke_copy3", "ke_naux", "ke_bc", "ke_ppe", "ke_step_post")

    def profile(self, enable: bool = True) -> None:
        """Per-stage CUDA-event timing of direct launches (graph replay is
        not profiled); enabling resets the sums."""
        self._check(self.L.wolfd2gpu_ens_profile(self.h, 1 if enable else 0))

    def profile_read(self, mixed: bool = True) -> dict:
        """Stage sums keyed by the kernel names of the mixed or plain step."""
        out = {}
        for k, name in enumerate(self.STAGES if mixed else self.STAGES_FP64):
            ms, n = C.c_double(), C.c_longlong()
            self._check(self.L.wolfd2gpu_ens_profile_read(self.h, k, C.byref(ms), C.byref(n)))
            out[name] = (ms.value, n.value)
        return out

    def graph(self, enable: bool) -> None:
        self.L.wolfd2gpu_ens_graph(self.h, 1 if enable else 0)

    def info(self) -> dict:
        bm, bp, ms, nl = C.c_int(), C.c_int(), C.c_double(), C.c_longlong()
        self._check(self.L.wolfd2gpu_ens_info(self.h, C.byref(bm), C.byref(bp), C.byref(ms), C.byref(nl)))
        return {"blocks_momentum": bm.value, "blocks_poisson": bp.value, "last_ms": ms.value,
                "launches": nl.value}

    def close(self) -> None:
        if getattr(self, "h", None):
            self.L.wolfd2gpu_ens_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
