"""CPU statement of the mixed-precision Ppe (TEST INFRASTRUCTURE ONLY).

The reference's Poisson solve is FP64 only; the mixed form has no
counterpart there.  It keeps the reference's red/black point iteration
(SorRB/SorRBP, src/pressure.f:457-656): black points (i+j even) first, then
red, relaxation factor sorrel, per-sweep dif = max |delta|, stop at the first
sweep m > 1 with dif < sortol or after msorit sweeps.  It runs that iteration
on the correction equation A e = r in FP32, where one refinement pass forms
r = b - A p in FP64, sweeps e from zero `inner` times (or until the stopping
rule fires), and adds e to p in FP64.  b = div/dk with the divergence of
src/pressure.f:287-299 (nloc = 1) and RhsPpe's Cartesian form
(src/pressure.f:354-359).

Every operation is stated in the order the GPU kernel evaluates it, in the
same IEEE type (numpy float32 elementwise arithmetic, no fused multiply-add),
and the points of one colour never read each other, so the GPU result is
expected to equal this model bit for bit.  The model's distance from the FP64
oracle is the accuracy figure of the mixed path.

``MixedRun`` advances a case in the order of main.f:690-972 with the mixed
form's precisions: nAuxMomentum in IEEE single (the oracle's FP32 instance of
its momentum restatement, on FP32 copies of u, v and of the metrics), the
mixed Ppe above, and the oracle's FP64 routines for the boundary rows, the
projection and the step norms.
"""
from __future__ import annotations

from typing import Dict, Optional

import numpy as np

from oracle import FIELD_NAMES, Oracle


def divergence(nx: int, ny: int, met: Dict[str, np.ndarray], u: np.ndarray, v: np.ndarray) -> np.ndarray:
    """Divergence nloc = 1 (src/pressure.f:287-299) on the pressure cells
    i = 2..nx, j = 2..ny, as an (nx-1, ny-1) array."""
    def s(a, di, dj):
        return a[2 + di:nx + 1 + di, 2 + dj:ny + 1 + dj]
    yeu, xeu, xzv, yzv = met["yeu"], met["xeu"], met["xzv"], met["yzv"]
    ucij = s(yeu, 0, 0) * s(u, 0, 0) - \
        s(xeu, 0, 0) * (s(v, 1, 0) + s(v, 0, 0) + s(v, 1, -1) + s(v, 0, -1)) / 4.0
    uci1j = s(yeu, -1, 0) * s(u, -1, 0) - \
        s(xeu, -1, 0) * (s(v, 0, 0) + s(v, -1, 0) + s(v, 0, -1) + s(v, -1, -1)) / 4.0
    vcij = s(xzv, 0, 0) * s(v, 0, 0) - \
        s(yzv, 0, 0) * (s(u, 0, 1) + s(u, -1, 1) + s(u, 0, 0) + s(u, -1, 0)) / 4.0
    vcij1 = s(xzv, 0, -1) * s(v, 0, -1) - \
        s(yzv, 0, -1) * (s(u, 0, 0) + s(u, -1, 0) + s(u, 0, -1) + s(u, -1, -1)) / 4.0
    return ucij - uci1j + vcij - vcij1


def div_check(nx: int, ny: int, met, u, v) -> float:
    """max |Divergence(u,v)| over the pressure cells (no blockages)."""
    return float(np.max(np.abs(divergence(nx, ny, met, u, v))))


def div_check_interior(nx: int, ny: int, met, u, v) -> float:
    """max |Divergence(u,v)| over the interior cells i, j = 3..n-1 (every
    neighbour an unknown of the Poisson equation; on a one-region layout
    also every face updated by Project), where the divergence is dk times
    the Poisson residual."""
    return float(np.max(np.abs(divergence(nx, ny, met, u, v)[1:-1, 1:-1])))


def ppe_rows(nx: int, ny: int, met):
    """The Poisson rows a1..a5 of pressure.f:97-106 on i, j = 2..nx, 2..ny,
    each an (nx-1, ny-1) array, a3 formed in the reference's order."""
    rau, rgv = met["rau"], met["rgv"]
    I, J, Im, Jm = slice(2, nx + 1), slice(2, ny + 1), slice(1, nx), slice(1, ny)
    a1, a2, a4, a5 = rgv[I, Jm], rau[Im, J], rau[I, J], rgv[I, J]
    a3 = -rau[I, J] - rau[Im, J] - rgv[I, J] - rgv[I, Jm]
    return a1, a2, a3, a4, a5


def is_unit_stencil(nx: int, ny: int, met) -> bool:
    """Every Poisson row is (1, 1, -4, 1, 1) (pressure.f:97-106)."""
    a1, a2, a3, a4, a5 = ppe_rows(nx, ny, met)
    return bool(np.all(a1 == 1.0) and np.all(a2 == 1.0) and np.all(a3 == -4.0) and
                np.all(a4 == 1.0) and np.all(a5 == 1.0))


def is_unit_stencil32(nx: int, ny: int, met) -> bool:
    """Every Poisson row rounds to (1, 1, -4, 1, 1) in FP32: the rows of any
    uniform square-cell Cartesian grid."""
    a = [x.astype(np.float32) for x in ppe_rows(nx, ny, met)]
    return bool(np.all(a[0] == 1) and np.all(a[1] == 1) and np.all(a[2] == -4) and
                np.all(a[3] == 1) and np.all(a[4] == 1))


def blockage_rows(nx: int, ny: int, regions) -> np.ndarray:
    """The cells whose Poisson row becomes the identity (0, 0, 1, 0, 0) and
    whose divergence is zeroed, by the blockage loops of pressure.f:109-196:
    a boolean (nx+2, ny+2) array indexed (i, j)."""
    idn = np.zeros((nx + 2, ny + 2), dtype=bool)
    if regions is None:
        return idn
    ni, nj = regions.n_i, regions.n_j
    blk = 0  # RM_BLOCKG
    W, E, S, N = 1, 2, 3, 4
    for jr in range(1, nj + 1):
        for ir in range(1, ni + 1):
            if regions.rtype(ir, jr) != blk:
                continue
            iw, ie = regions.border(ir, jr, W), regions.border(ir, jr, E)
            js, jn = regions.border(ir, jr, S), regions.border(ir, jr, N)
            idn[iw + 2:ie, js + 2:jn] = True
            if ir > 1 and regions.rtype(ir - 1, jr) == blk:
                idn[iw + 1, js + 1:jn + 1] = True
            if ir < ni and regions.rtype(ir + 1, jr) == blk:
                idn[ie, js + 1:jn + 1] = True
            if jr > 1 and regions.rtype(ir, jr - 1) == blk:
                idn[iw + 1:ie + 1, js + 1] = True
            if jr < nj and regions.rtype(ir, jr + 1) == blk:
                idn[iw + 1:ie + 1, jn] = True
    return idn


def _cross(nx: int, ny: int, rbu, rbv, P):
    """RhsPpe's non-Cartesian cross terms (src/pressure.f:360-375) on the
    unknowns, in its operand order and in the type of P and the metric
    arrays: rbu(i,j) (...) - rbu(i-1,j) (...) + rbv(i,j) (...) - rbv(i,j-1) (...)."""
    def s(a, di, dj):
        return a[2 + di:nx + 1 + di, 2 + dj:ny + 1 + dj]
    return (s(rbu, 0, 0) * (s(P, 1, 1) + s(P, 0, 1) - s(P, 1, -1) - s(P, 0, -1)) -
            s(rbu, -1, 0) * (s(P, 0, 1) + s(P, -1, 1) - s(P, 0, -1) - s(P, -1, -1)) +
            s(rbv, 0, 0) * (s(P, 1, 1) + s(P, 1, 0) - s(P, -1, 1) - s(P, -1, 0)) -
            s(rbv, 0, -1) * (s(P, 1, 0) + s(P, 1, -1) - s(P, -1, 0) - s(P, -1, -1)))


def ppe_mixed_general(nx: int, ny: int, met, u, v, p, dk: float, msorit: int, sortol: float,
                      sorrel: float, inner: int, regions=None, lcartes: int = 1) -> int:
    """Mixed Ppe with the grid's own Poisson rows in the FP32 sweeps: any
    Cartesian grid (cells of any shape and spacing, blockage identity rows)
    and, with lcartes = 0, curvilinear grids.

    Each refinement pass forms r = RhsPpe(p) - A p in FP64 with the rows of
    pressure.f:97-196 (RhsPpe's cross terms of the current p when lcartes =
    0), then relaxes A e = r from e = 0 in FP32 with the rows rounded to
    FP32 (c_k = a_k): per sweep (lcartes = 0: r' = r - the cross terms of e
    in FP32, with rbu, rbv rounded to FP32, formed before the sweep as the
    reference forms its right-hand side), black points then red,
    s = r' - c1 eS - c2 eW - c4 eE - c5 eN, s = s * (1/c3) - e,
    e = e + sorrel s, dif = max |s|, where 1/c3 is the FP32 reciprocal of
    the rounded diagonal (the reference divides, pressure.f:437; a product
    by the reciprocal is one rounding of a different operator, which the
    FP64 residual of the next pass corrects like any FP32 error).  Stopping
    rule and pass lengths as ppe_mixed.  On unit rows every operation
    equals the unit form's bit for bit (1 x == x, 1/-4 == -0.25 exactly)."""
    f32 = np.float32
    a1, a2, a3, a4, a5 = (a.copy() for a in ppe_rows(nx, ny, met))
    idn = blockage_rows(nx, ny, regions)[2:nx + 1, 2:ny + 1]
    for a in (a1, a2, a4, a5):
        a[idn] = 0.0
    a3[idn] = 1.0
    div = divergence(nx, ny, met, u, v)
    div[idn] = 0.0
    b = div / dk
    c1, c2, c3, c4, c5 = (a.astype(f32) for a in (a1, a2, a3, a4, a5))
    rc3 = f32(1.0) / c3
    rbu32, rbv32 = met["rbu"].astype(f32), met["rbv"].astype(f32)
    I, J = np.meshgrid(np.arange(2, nx + 1), np.arange(2, ny + 1), indexing="ij")
    cols = []
    for c in (0, 1):
        sel = ((I + J) & 1) == c
        cols.append((I[sel], J[sel], sel))
    relax = f32(sorrel)
    m = 0
    result = 0
    done = False
    while not done:
        ps = p[2:nx + 1, 2:ny + 1]
        bb = b if lcartes else b - _cross(nx, ny, met["rbu"], met["rbv"], p)
        ap = (a1 * p[2:nx + 1, 1:ny] + a2 * p[1:nx, 2:ny + 1] + a4 * p[3:nx + 2, 2:ny + 1] +
              a5 * p[2:nx + 1, 3:ny + 2] + a3 * ps)
        R = (bb - ap).astype(f32)
        E = np.zeros((nx + 2, ny + 2), dtype=f32)
        in_pass = 0
        while True:
            m += 1
            RR = R if lcartes else R - _cross(nx, ny, rbu32, rbv32, E)
            dif = f32(0.0)
            for ii, jj, sel in cols:
                c0 = E[ii, jj]
                s = RR[sel] - c1[sel] * E[ii, jj - 1] - c2[sel] * E[ii - 1, jj] - \
                    c4[sel] * E[ii + 1, jj] - c5[sel] * E[ii, jj + 1]
                s = s * rc3[sel] - c0
                E[ii, jj] = c0 + relax * s
                if s.size:
                    dif = max(dif, np.max(np.abs(s)))
            if m > 1 and float(dif) < sortol:
                result = m
                done = True
                break
            in_pass += 1
            if m >= msorit:
                done = True
                break
            if in_pass >= inner:
                break
        p[2:nx + 1, 2:ny + 1] = ps + E[2:nx + 1, 2:ny + 1].astype(np.float64)
    return result if result >= 1 else msorit


def ppe_mixed(nx: int, ny: int, met, u, v, p, dk: float, msorit: int, sortol: float,
              sorrel: float, inner: int, dtype=np.float32) -> int:
    """Mixed Ppe on a Cartesian grid without blockages whose Poisson rows
    round to the unit stencil in FP32; p is updated in place on i = 2..nx,
    j = 2..ny.  The FP32 sweeps run the unit stencil, each pass's FP64
    residual the grid's own rows (the unit form when they are exactly
    unit).  Returns nSorConv (msorit when the stopping rule never fired).
    dtype = float64 gives the same iteration with FP64 sweeps."""
    if not is_unit_stencil32(nx, ny, met):
        raise ValueError("mixed Ppe needs rows that round to the unit stencil in FP32")
    unit = is_unit_stencil(nx, ny, met)
    a1, a2, a3, a4, a5 = ppe_rows(nx, ny, met)
    b = divergence(nx, ny, met, u, v) / dk
    I, J = np.meshgrid(np.arange(2, nx + 1), np.arange(2, ny + 1), indexing="ij")
    cols = []
    for c in (0, 1):
        sel = ((I + J) & 1) == c
        cols.append((I[sel], J[sel]))
    relax = dtype(sorrel)
    quarter = dtype(-0.25)
    m = 0
    result = 0
    done = False
    while not done:
        ps = p[2:nx + 1, 2:ny + 1]
        if unit:
            ap = p[2:nx + 1, 1:ny] + p[1:nx, 2:ny + 1] + p[3:nx + 2, 2:ny + 1] + p[2:nx + 1, 3:ny + 2] - 4.0 * ps
        else:
            ap = (a1 * p[2:nx + 1, 1:ny] + a2 * p[1:nx, 2:ny + 1] + a4 * p[3:nx + 2, 2:ny + 1] +
                  a5 * p[2:nx + 1, 3:ny + 2] + a3 * ps)
        R = np.zeros((nx + 2, ny + 2), dtype=dtype)
        R[2:nx + 1, 2:ny + 1] = (b - ap).astype(dtype)
        E = np.zeros((nx + 2, ny + 2), dtype=dtype)
        in_pass = 0
        while True:
            m += 1
            dif = dtype(0.0)
            for ii, jj in cols:
                c0 = E[ii, jj]
                s = R[ii, jj] - E[ii, jj - 1] - E[ii - 1, jj] - E[ii + 1, jj] - E[ii, jj + 1]
                s = s * quarter - c0
                E[ii, jj] = c0 + relax * s
                if s.size:
                    dif = max(dif, np.max(np.abs(s)))
            if m > 1 and float(dif) < sortol:
                result = m
                done = True
                break
            in_pass += 1
            if m >= msorit:
                done = True
                break
            if in_pass >= inner:
                break
        p[2:nx + 1, 2:ny + 1] = ps + E[2:nx + 1, 2:ny + 1].astype(np.float64)
    return result if result >= 1 else msorit


class MixedRun:
    """A case advanced by the time loop of main.f:690-972 with the mixed
    Ppe in place of the FP64 one; ``history`` holds (nQLiter, nSorConv,
    dif(1..4), divmax, divmax over the interior cells) per step."""

    def __init__(self, case, fields: Optional[Dict[str, np.ndarray]] = None, cold_start: bool = True,
                 inner: int = 64):
        self.case = case
        self.nx, self.ny = case.nx, case.ny
        self.prm = case.params
        self.inner = inner
        self.o = Oracle(case.nx + 1, case.ny + 1)
        self.met = self.o.grid(case.nx, case.ny, case.x, case.y)
        self.met32 = self.o.metrics32(self.met)
        self.f = {n: self.o.field() for n in FIELD_NAMES}
        if fields:
            for k, val in fields.items():
                self.f[k][...] = val
        self.history = []
        self.cold_nconv = None
        # the unit-stencil sweeps where every row rounds to it in FP32 on a
        # Cartesian grid without blockages, else the grid's own rows
        self.general = not (self.prm.lcartes and is_unit_stencil32(self.nx, self.ny, self.met) and
                            not blockage_rows(self.nx, self.ny, case.regions).any())
        if cold_start:
            f, o, nx, ny, r = self.f, self.o, self.nx, self.ny, case.regions
            o.vel_bound_cond(nx, ny, r, f["u"], f["v"])
            self.cold_nconv = self._ppe(f["u"], f["v"], f["p"])
            o.pres_bound_cond(nx, ny, r, f["p"])
            o.project(nx, ny, r, self.prm.dk, self.met, f["p"], f["u"], f["v"])
            o.vel_bound_cond(nx, ny, r, f["u"], f["v"])

    def _ppe(self, u, v, p) -> int:
        prm = self.prm
        if self.general:
            return ppe_mixed_general(self.nx, self.ny, self.met, u, v, p, prm.dk, prm.msorit, prm.sortol,
                                     prm.sorrel, self.inner, regions=self.case.regions, lcartes=prm.lcartes)
        return ppe_mixed(self.nx, self.ny, self.met, u, v, p, prm.dk, prm.msorit, prm.sortol,
                         prm.sorrel, self.inner)

    def step(self, n: int = 1):
        f, o, nx, ny, r, prm = self.f, self.o, self.nx, self.ny, self.case.regions, self.prm
        for _ in range(n):
            for a, b in (("pn", "p"), ("un", "u"), ("vn", "v"), ("us", "u"), ("vs", "v")):
                f[a][...] = f[b]
            un32 = np.asfortranarray(f["un"].astype(np.float32))
            vn32 = np.asfortranarray(f["vn"].astype(np.float32))
            us32, vs32, z32 = un32.copy(order="F"), vn32.copy(order="F"), o.field32()
            nql = o.naux_momentum_f32(nx, ny, r, prm, self.met32, z32, z32, un32, vn32, us32, vs32)
            f["us"][...] = us32.astype(np.float64)
            f["vs"][...] = vs32.astype(np.float64)
            if prm.nfiltu == 1:
                o.filter(nx, ny, 1, r, prm.fpu, f["us"])
            if prm.nfiltv == 1:
                o.filter(nx, ny, 2, r, prm.fpv, f["vs"])
            o.vel_bound_cond(nx, ny, r, f["us"], f["vs"])
            o.pres_bound_cond(nx, ny, r, f["p"])
            nsor = self._ppe(f["us"], f["vs"], f["p"])
            o.pres_bound_cond(nx, ny, r, f["p"])
            o.project(nx, ny, r, prm.dk, self.met, f["p"], f["us"], f["vs"])
            o.vel_bound_cond(nx, ny, r, f["us"], f["vs"])
            o.pres_bound_cond(nx, ny, r, f["p"])
            f["u"][...] = f["us"]
            f["v"][...] = f["vs"]
            o.vel_bound_cond(nx, ny, r, f["u"], f["v"])
            o.pres_bound_cond(nx, ny, r, f["p"])
            dif = (o.diff_max_norm(nx, ny, f["pn"], f["p"]), o.diff_max_norm(nx, ny, f["un"], f["u"]),
                   o.diff_max_norm(nx, ny, f["vn"], f["v"]), 0.0)
            self.history.append((nql, nsor, dif, div_check(nx, ny, self.met, f["u"], f["v"]),
                                 div_check_interior(nx, ny, self.met, f["u"], f["v"])))
            if max(dif) > 1.0e12:
                raise FloatingPointError("Solution diverged. Please reduce CFL number.")
        return self.history[-1]
