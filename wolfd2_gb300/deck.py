"""Host-side case setup: region tables, boundary-condition tables and run
parameters in the reference's own Fortran layouts.

This mirrors the part of the reference's input layer that produces the hot
path's inputs:

* ``boundary_conditions`` keywords ``number_of_regions``, ``i_borders``,
  ``j_borders``, ``wall``, ``inlet``, ``outlet``, ``blockage`` and ``porous_region``
  (src/parse.f:1005-1950), defaults from ``InitBCFlags`` (src/parse.f:2257-2380);
* the region-border fill and boundary-type consistency passes of
  ``SetUpBCs`` (src/bound_cond.f:123-223) and the porous constants of
  ``PorRegCnst`` (src/bound_cond.f:1883-1986);
* the input-parameter defaults (src/parse.f:117-193) and the
  Reynolds/Froude/time-step scaling of ``ReadParam``
  (src/file_manip.f:130-157).

Tables are numpy arrays with Fortran (column-major) order and the
reference's shapes (mgri=20, mgrj=10 from include/config.f), so the same
buffers can be handed to the C-ABI exactly as the Fortran driver would.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

# include/config.f:19-26
MGRI = 20
MGRJ = 10

# include/wolfd2.h:15-60
RM_BLOCKG, RM_INTERN, RM_POROUS = 0, 1, 2
BM_INTERN, BM_WALL1, BM_WALL2, BM_INLET, BM_OUTLT1, BM_OUTLT2 = 0, 1, 2, 3, 4, 5
WEST, EAST, SOUTH, NORTH = 1, 2, 3, 4
VAR_U, VAR_V, VAR_P, VAR_T = 1, 2, 3, 4

# ppe_solver keywords, src/parse.f:449-460
PPE_SOLVERS = {"sor": 1, "lsor": 2, "rb_lsor": 3, "par_rb_lsor": 4,
               "rb_sor": 5, "par_rb_sor": 6}

_FACES = {"w": WEST, "west": WEST, "e": EAST, "east": EAST,
          "s": SOUTH, "south": SOUTH, "n": NORTH, "north": NORTH}


@dataclasses.dataclass
class Regions:
    """Region/boundary tables in Fortran layout (1-based meaning, 0-based
    storage: element (ireg,jreg,face) lives at [ireg-1, jreg-1, face-1])."""
    nReg: np.ndarray          # int32 (2,)
    nRegBrd: np.ndarray       # int32 (mgri, mgrj, 4)
    nRegType: np.ndarray      # int32 (mgri, mgrj)
    nMomBdTp: np.ndarray      # int32 (mgri, mgrj, 4)
    dBCVal: np.ndarray        # float64 (mgri, mgrj, 4, 4)
    dPRporos: np.ndarray      # float64 (mgri, mgrj)
    dPRporc1: np.ndarray
    dPRporc2: np.ndarray
    # Per-position face values (an extension: the reference's faces carry one
    # constant per variable): {(ireg, jreg, face, var): values}, var 1 = u,
    # 2 = v, values[pos] at position pos along the face (j on west/east
    # faces, i on south/north faces); they replace dBCVal in VelBoundCond's
    # inlet and moving-wall rows.
    profiles: dict = dataclasses.field(default_factory=dict)
    # thermal tables of the same section (parse.f's thermal keywords); face
    # temperatures are dBCVal(..., VAR_T)
    thermal: Optional["Thermal"] = None

    @property
    def n_i(self) -> int:
        return int(self.nReg[0])

    @property
    def n_j(self) -> int:
        return int(self.nReg[1])

    def border(self, ireg: int, jreg: int, face: int) -> int:
        return int(self.nRegBrd[ireg - 1, jreg - 1, face - 1])

    def btype(self, ireg: int, jreg: int, face: int) -> int:
        return int(self.nMomBdTp[ireg - 1, jreg - 1, face - 1])

    def rtype(self, ireg: int, jreg: int) -> int:
        return int(self.nRegType[ireg - 1, jreg - 1])


def _empty_tables() -> Regions:
    f = dict(order="F")
    return Regions(
        nReg=np.zeros(2, np.int32),
        nRegBrd=np.zeros((MGRI, MGRJ, 4), np.int32, **f),
        nRegType=np.zeros((MGRI, MGRJ), np.int32, **f),
        nMomBdTp=np.zeros((MGRI, MGRJ, 4), np.int32, **f),
        dBCVal=np.zeros((MGRI, MGRJ, 4, 4), np.float64, **f),
        dPRporos=np.zeros((MGRI, MGRJ), np.float64, **f),
        dPRporc1=np.zeros((MGRI, MGRJ), np.float64, **f),
        dPRporc2=np.zeros((MGRI, MGRJ), np.float64, **f),
    )


class DeckError(ValueError):
    """A boundary-condition or parameter deck the reference would reject."""


def _init_bc_flags(t: Regions) -> None:
    """InitBCFlags, src/parse.f:2257-2380: momentum and temperature."""
    ni, nj = t.n_i, t.n_j
    t.dBCVal[:ni, :nj, :, :] = 0.0
    t.nRegType[:ni, :nj] = RM_INTERN
    t.nMomBdTp[:ni, :nj, :] = BM_INTERN
    t.nMomBdTp[0, :nj, WEST - 1] = BM_WALL1
    t.nMomBdTp[ni - 1, :nj, EAST - 1] = BM_WALL1
    t.nMomBdTp[:ni, 0, SOUTH - 1] = BM_WALL1
    t.nMomBdTp[:ni, nj - 1, NORTH - 1] = BM_WALL1
    # temperature: no sources, interfaces inside, adiabatic outer walls
    th = t.thermal
    th.nTRgType[:ni, :nj] = RT_NOSRCE
    th.nTemBdTp[:ni, :nj, :] = BT_INTERN
    th.nTemBdTp[0, :nj, WEST - 1] = BT_HTFLUX
    th.nTemBdTp[ni - 1, :nj, EAST - 1] = BT_HTFLUX
    th.nTemBdTp[:ni, 0, SOUTH - 1] = BT_HTFLUX
    th.nTemBdTp[:ni, nj - 1, NORTH - 1] = BT_HTFLUX


def parse_bc_section(text: str, nx: int, ny: int, *, uref: float = 1.0,
                     densref: float = 1.0, dlref: float = 1.0,
                     re: float = 1.0, tref: float = 0.0, tmax: float = 1.0) -> Regions:
    """Parse a ``boundary_conditions`` section body (lines between
    ``section boundary_conditions`` and ``end section``) and run the
    ``SetUpBCs`` passes.  Keywords are case-insensitive; ``#`` starts a
    comment (src/parse.f:1168-1210).  Temperatures are scaled to
    (T - tref) / (tmax - tref) (src/parse.f:1366, 1565, 1834); the thermal
    tables land in ``Regions.thermal`` (heat generation values stay as read:
    :func:`heat_sources` scales them)."""
    t = _empty_tables()
    t.thermal = Thermal.empty()
    th = t.thermal

    def temp_of(word: str) -> float:
        try:
            return (float(word) - tref) / (tmax - tref)
        except ValueError as exc:
            raise DeckError(f"expected a temperature, got {word!r}") from exc

    def fixed_temperature(ir: int, jr: int, val: float, neighbours: bool) -> None:
        """A fixed-temperature region: its faces (and with `neighbours` the
        coinciding faces of its neighbours) at that temperature."""
        i0, j0 = ir - 1, jr - 1
        th.nTRgType[i0, j0] = RT_TEMPER
        th.dTRgVal[i0, j0] = val
        th.nTemBdTp[i0, j0, :] = BT_TEMPER
        t.dBCVal[i0, j0, :, VAR_T - 1] = val
        if not neighbours:
            return
        for di, dj, face in ((-1, 0, EAST), (1, 0, WEST), (0, -1, NORTH), (0, 1, SOUTH)):
            a, b = i0 + di, j0 + dj
            if 0 <= a < t.n_i and 0 <= b < t.n_j:
                th.nTemBdTp[a, b, face - 1] = BT_TEMPER
                t.dBCVal[a, b, face - 1, VAR_T - 1] = val
    found_nreg = def_i = def_j = False
    perm_eq = np.zeros((MGRI, MGRJ), np.int32, order="F")
    dim_coef = np.zeros((MGRI, MGRJ, 3), np.float64, order="F")

    def need_ij(words: List[str], k: int) -> Tuple[int, int]:
        try:
            ir, jr = int(words[k]), int(words[k + 1])
        except (IndexError, ValueError) as exc:
            raise DeckError(f"expected region indices in {' '.join(words)!r}") from exc
        if not (1 <= ir <= MGRI and 1 <= jr <= MGRJ):
            raise DeckError(f"region index out of range: {ir},{jr}")
        return ir, jr

    def face_of(word: str) -> int:
        if word not in _FACES:
            raise DeckError(f"Unrecognized cell face designation: [{word}]")
        return _FACES[word]

    for raw in text.splitlines():
        line = raw.split("#", 1)[0].strip().lower()
        if not line:
            continue
        w = line.split()
        key = w[0]
        if key == "number_of_regions":
            ir, jr = need_ij(w, 1)
            t.nReg[:] = (ir, jr)
            found_nreg = True
        elif key == "i_borders":
            if not found_nreg:
                raise DeckError("Error: Number_of_Regions not defined")
            vals = [int(x) for x in w[1:]]
            if len(vals) < t.n_i - 1:
                raise DeckError("i_borders: too few values")
            for k in range(2, t.n_i + 1):
                t.nRegBrd[k - 1, 0, WEST - 1] = vals[k - 2]
            def_i = True
            if def_j:
                _init_bc_flags(t)
        elif key == "j_borders":
            if not found_nreg:
                raise DeckError("Error: Number_of_Regions not defined")
            vals = [int(x) for x in w[1:]]
            if len(vals) < t.n_j - 1:
                raise DeckError("j_borders: too few values")
            for k in range(2, t.n_j + 1):
                t.nRegBrd[0, k - 1, SOUTH - 1] = vals[k - 2]
            def_j = True
            if def_i:
                _init_bc_flags(t)
        elif key == "blockage":
            ir, jr = need_ij(w, 1)
            t.nRegType[ir - 1, jr - 1] = RM_BLOCKG
            t.nMomBdTp[ir - 1, jr - 1, :] = BM_WALL1
            th.nTemBdTp[ir - 1, jr - 1, :] = BT_HTFLUX
            if ir > 1:
                t.nMomBdTp[ir - 2, jr - 1, EAST - 1] = BM_WALL1
                th.nTemBdTp[ir - 2, jr - 1, EAST - 1] = BT_HTFLUX
            if ir < t.n_i:
                t.nMomBdTp[ir, jr - 1, WEST - 1] = BM_WALL1
                th.nTemBdTp[ir, jr - 1, WEST - 1] = BT_HTFLUX
            if jr > 1:
                t.nMomBdTp[ir - 1, jr - 2, NORTH - 1] = BM_WALL1
                th.nTemBdTp[ir - 1, jr - 2, NORTH - 1] = BT_HTFLUX
            if jr < t.n_j:
                t.nMomBdTp[ir - 1, jr, SOUTH - 1] = BM_WALL1
                th.nTemBdTp[ir - 1, jr, SOUTH - 1] = BT_HTFLUX
            # src/parse.f:1347-1400: "temper <T>" makes it a fixed-temperature block
            k = 3
            while k < len(w):
                if w[k] in ("temper", "t") and k + 1 < len(w):
                    fixed_temperature(ir, jr, temp_of(w[k + 1]), True)
                    k += 2
                else:
                    raise DeckError(f"blockage: unrecognized word {w[k]!r}")
        elif key == "porous_region":
            ir, jr = need_ij(w, 1)
            t.nRegType[ir - 1, jr - 1] = RM_POROUS
            # permeability equation names, src/parse.f:1422-1432
            eqs = {"carman-kozeny": 1, "kaviany": 2, "happen-brenner": 3}
            if len(w) < 7 or w[3] not in eqs:
                raise DeckError(f"porous: bad syntax {line!r}")
            perm_eq[ir - 1, jr - 1] = eqs[w[3]]
            dim_coef[ir - 1, jr - 1, :] = [float(x) for x in w[4:7]]
        elif key in ("wall", "inlet", "outlet"):
            ir, jr = need_ij(w, 1)
            if len(w) < 4:
                raise DeckError(f"{key}: missing face")
            face = face_of(w[3])
            rest = w[4:]
            i0, j0 = ir - 1, jr - 1
            if key == "wall":
                t.nMomBdTp[i0, j0, face - 1] = BM_WALL1
            elif key == "inlet":
                t.nMomBdTp[i0, j0, face - 1] = BM_INLET
                if not rest:
                    raise DeckError("inlet: needs at least one value")
            else:
                t.nMomBdTp[i0, j0, face - 1] = BM_OUTLT2
            k = 0
            while k < len(rest):
                word = rest[k]
                if key == "wall" and word == "no_slip":
                    t.nMomBdTp[i0, j0, face - 1] = BM_WALL1
                elif key == "wall" and word == "no_stress":
                    t.nMomBdTp[i0, j0, face - 1] = BM_WALL2
                elif key == "outlet" and word in ("fully_dev", "fd"):
                    t.nMomBdTp[i0, j0, face - 1] = BM_OUTLT1
                elif key == "outlet" and word in ("mass_cons", "mc"):
                    t.nMomBdTp[i0, j0, face - 1] = BM_OUTLT2
                elif key != "outlet" and word in ("tangent_vel", "tv", "normal_vel", "nv"):
                    val = float(rest[k + 1]) / uref
                    normal = word in ("normal_vel", "nv")
                    if key == "wall" and normal:
                        raise DeckError("wall: normal velocity not allowed")
                    ew = face in (WEST, EAST)
                    var = (VAR_U if ew else VAR_V) if normal else (VAR_V if ew else VAR_U)
                    t.dBCVal[i0, j0, face - 1, var - 1] = val
                    k += 1
                elif key != "inlet" and word in ("press", "p"):
                    t.dBCVal[i0, j0, face - 1, VAR_P - 1] = float(rest[k + 1]) / (densref * uref * uref)
                    k += 1
                elif word in ("temper", "t"):
                    if k + 1 >= len(rest):
                        raise DeckError(f"{key}: temperature value missing")
                    th.nTemBdTp[i0, j0, face - 1] = BT_TEMPER
                    t.dBCVal[i0, j0, face - 1, VAR_T - 1] = temp_of(rest[k + 1])
                    k += 1
                else:
                    raise DeckError(f"{key}: unrecognized word {word!r}")
                k += 1
        elif key == "heat_generation_region":
            ir, jr = need_ij(w, 1)
            if len(w) < 4:
                raise DeckError("heat_generation_region: value missing")
            th.nTRgType[ir - 1, jr - 1] = RT_HEATGN
            th.dTRgVal[ir - 1, jr - 1] = float(w[3])
        elif key == "fixed_temperature_region":
            ir, jr = need_ij(w, 1)
            if len(w) < 4:
                raise DeckError("fixed_temperature_region: value missing")
            fixed_temperature(ir, jr, temp_of(w[3]), False)
        elif key in ("fixed_temperature_wall", "heat_flux_wall"):
            ir, jr = need_ij(w, 1)
            if len(w) < 4:
                raise DeckError(f"{key}: missing face")
            face = face_of(w[3])
            if key == "heat_flux_wall":
                # only adiabatic walls (src/parse.f:1924-1926)
                th.nTemBdTp[ir - 1, jr - 1, face - 1] = BT_HTFLUX
            else:
                if len(w) < 5:
                    raise DeckError("fixed_temperature_wall: value missing")
                th.nTemBdTp[ir - 1, jr - 1, face - 1] = BT_TEMPER
                t.dBCVal[ir - 1, jr - 1, face - 1, VAR_T - 1] = temp_of(w[4])
        else:
            raise DeckError(f"Unrecognized keyword: [{key}]")

    if not (found_nreg and def_i and def_j):
        raise DeckError("number_of_regions, i_borders and j_borders are required")
    _setup_bcs(t, nx, ny)
    _por_reg_cnst(t, perm_eq, dim_coef, dlref, re)
    return t


def _setup_bcs(t: Regions, nx: int, ny: int) -> None:
    """Border checks, border fill and type consistency,
    src/bound_cond.f:123-223."""
    ni, nj = t.n_i, t.n_j
    B = t.nRegBrd
    for ir in range(2, ni + 1):
        b = B[ir - 1, 0, WEST - 1]
        if b < 2 or b > nx - 2:
            raise DeckError(f"Bad iRegW index: {b}. Must be >= 2 and <= nx-2.")
    for ir in range(2, ni):
        if B[ir, 0, WEST - 1] - B[ir - 1, 0, WEST - 1] < 2:
            raise DeckError("i borders must increase by at least 2")
    for jr in range(2, nj + 1):
        b = B[0, jr - 1, SOUTH - 1]
        if b < 2 or b > ny - 2:
            raise DeckError(f"Bad jRegS index: {b}. Must be >= 2 and <= ny-2")
    for jr in range(2, nj):
        if B[0, jr, SOUTH - 1] - B[0, jr - 1, SOUTH - 1] < 2:
            raise DeckError("j borders must increase by at least 2")
    for jr in range(nj):
        B[0, jr, WEST - 1] = 1
        B[ni - 1, jr, EAST - 1] = nx
    for ir in range(ni):
        B[ir, 0, SOUTH - 1] = 1
        B[ir, nj - 1, NORTH - 1] = ny
    for jr in range(1, nj):
        for ir in range(1, ni):
            B[ir, jr, WEST - 1] = B[ir, 0, WEST - 1]
            B[ir, jr, SOUTH - 1] = B[0, jr, SOUTH - 1]
    for jr in range(nj):
        for ir in range(ni - 1):
            B[ir, jr, EAST - 1] = B[ir + 1, 0, WEST - 1]
    for jr in range(nj - 1):
        for ir in range(ni):
            B[ir, jr, NORTH - 1] = B[0, jr + 1, SOUTH - 1]
    T = t.nMomBdTp
    for jr in range(nj):
        for ir in range(ni - 1):
            if T[ir, jr, EAST - 1] == BM_INLET:
                T[ir + 1, jr, WEST - 1] = BM_INLET
            if T[ir + 1, jr, WEST - 1] == BM_INLET:
                T[ir, jr, EAST - 1] = BM_INLET
            if T[ir, jr, EAST - 1] == BM_WALL1:
                T[ir + 1, jr, WEST - 1] = BM_WALL1
            if T[ir + 1, jr, WEST - 1] == BM_WALL1:
                T[ir, jr, EAST - 1] = BM_WALL1
    for jr in range(nj - 1):
        for ir in range(ni):
            if T[ir, jr + 1, SOUTH - 1] == BM_INLET:
                T[ir, jr, NORTH - 1] = BM_INLET
            if T[ir, jr, NORTH - 1] == BM_INLET:
                T[ir, jr + 1, SOUTH - 1] = BM_INLET
            if T[ir, jr + 1, SOUTH - 1] == BM_WALL1:
                T[ir, jr, NORTH - 1] = BM_WALL1
            if T[ir, jr, NORTH - 1] == BM_WALL1:
                T[ir, jr + 1, SOUTH - 1] = BM_WALL1
    if t.thermal is None:
        return
    # the same pairing of coinciding faces for temperature (src/bound_cond.f:226-258)
    Q = t.thermal.nTemBdTp
    for jr in range(nj):
        for ir in range(ni - 1):
            for bt in (BT_TEMPER, BT_HTFLUX):
                if Q[ir, jr, EAST - 1] == bt:
                    Q[ir + 1, jr, WEST - 1] = bt
                if Q[ir + 1, jr, WEST - 1] == bt:
                    Q[ir, jr, EAST - 1] = bt
    for jr in range(nj - 1):
        for ir in range(ni):
            for bt in (BT_TEMPER, BT_HTFLUX):
                if Q[ir, jr + 1, SOUTH - 1] == bt:
                    Q[ir, jr, NORTH - 1] = bt
                if Q[ir, jr, NORTH - 1] == bt:
                    Q[ir, jr + 1, SOUTH - 1] = bt


def heat_sources(regions: Regions, dlref: float, tref: float, tmax: float, dconduct: float,
                 pe: float) -> None:
    """dHGSTval of the heat-generating regions from the values the deck gave
    (src/bound_cond.f:2018-2029): s = q dlref^2 / (pe dconduct (tmax - tref))."""
    th = regions.thermal
    for jr in range(regions.n_j):
        for ir in range(regions.n_i):
            if th.nTRgType[ir, jr] == RT_HEATGN:
                th.dHGSTval[ir, jr] = (th.dTRgVal[ir, jr] * dlref ** 2) / (pe * dconduct * (tmax - tref))


def _por_reg_cnst(t: Regions, perm_eq, dim_coef, dlref: float, re: float) -> None:
    """PorRegCnst, src/bound_cond.f:1883-1986."""
    dpi4 = math.acos(-1.0) / 4.0
    for jr in range(t.n_j):
        for ir in range(t.n_i):
            if t.nRegType[ir, jr] != RM_POROUS:
                t.dPRporos[ir, jr] = 1.0
                t.dPRporc1[ir, jr] = 0.0
                t.dPRporc2[ir, jr] = 0.0
                continue
            por, dia, cf = (float(x) for x in dim_coef[ir, jr])
            if (1.0 - por) < 1.0e-4:
                por = 0.98
            eq = int(perm_eq[ir, jr])
            if eq == 1:
                perm = (dia ** 2 * por ** 3) / (1.8e2 * (1.0 - por) ** 2)
            elif eq == 2:
                perm = 0.0606 * dpi4 * (por ** 5.10) * dia ** 2 / (1.0 - por)
            elif eq == 3:
                pors = 1.0 - por
                pors2 = pors ** 2
                koz = (2.0 * por ** 3) / pors / (math.log(1.0 / pors) - (1.0 - pors2) / (1.0 + pors2))
                perm = dia ** 2 * por ** 3 / (16.0 * koz * pors2)
            else:
                raise DeckError("Wrong nPermEq flag")
            t.dPRporos[ir, jr] = float(dim_coef[ir, jr, 0])
            t.dPRporc1[ir, jr] = (por * dlref ** 2) / (re * perm)
            t.dPRporc2[ir, jr] = (dlref * cf * por) / math.sqrt(perm)


@dataclasses.dataclass
class RunParams:
    """Time-loop parameters after ReadParam's scaling (nthermen = 0)."""
    dk: float                   # dimensionless time step (dk*uref/dlref)
    re: float
    fr: float
    nts: int = 0
    mqiter: int = 20            # src/parse.f:135-148 defaults
    qtol: float = 1.0e-4
    npsolver: int = 1
    msorit: int = 2000
    sortol: float = 1.0e-8
    sorrel: float = 1.0
    nfiltu: int = 0
    nfiltv: int = 0
    fpu: float = 5.0e2
    fpv: float = 5.0e2
    lcartes: int = 0

    @staticmethod
    def scaled(dt: float, dlref: float, uref: float, rho: float, mu: float,
               **kw) -> "RunParams":
        """ReadParam scaling, src/file_manip.f:130-157."""
        kinvisc = mu / rho
        re = dlref * uref / kinvisc
        fr = uref ** 2.0 / (dlref * 9.81)
        return RunParams(dk=dt * uref / dlref, re=re, fr=fr, **kw)


# include/wolfd2.h: thermal region and boundary types
RT_NOSRCE, RT_HEATGN, RT_TEMPER = 0, 1, 2
BT_INTERN, BT_TEMPER, BT_HTFLUX = 0, 1, 2


@dataclasses.dataclass
class Thermal:
    """Thermal region/boundary tables of ThermEnergy and TempBoundCond
    (src/thermal.f:24-73, src/bound_cond.f:1030-1063), Fortran layout like
    Regions; face temperatures are dBCVal(..., VAR_T)."""
    nTRgType: np.ndarray      # int32 (mgri, mgrj): RT_*
    nTemBdTp: np.ndarray      # int32 (mgri, mgrj, 4): BT_*
    dTRgVal: np.ndarray       # float64 (mgri, mgrj): fixed-region temperature
    dHGSTval: np.ndarray      # float64 (mgri, mgrj): heat generation source

    @classmethod
    def empty(cls) -> "Thermal":
        f = dict(order="F")
        return cls(np.zeros((MGRI, MGRJ), np.int32, **f), np.zeros((MGRI, MGRJ, 4), np.int32, **f),
                   np.zeros((MGRI, MGRJ), np.float64, **f), np.zeros((MGRI, MGRJ), np.float64, **f))


@dataclasses.dataclass
class SmallScaleParams:
    """Switch and constants of the small-scale (ATD) model, SmallScale
    (src/small_scale.f:31-578), with ReadParam's defaults (src/parse.f:
    144-178): its own Ppe solver and sweep limit, the chaotic-map constants
    and the Shuman filter parameters of u, v and t.  SmallScale also reads
    dlref, uref, tref, tmax and pe (pe / re is its Prandtl number); it
    always takes the thermal tables of the case (TempBoundCond, Filter of t)."""
    npsolver: int = 1           # nssPpeSlvr
    msorit: int = 2000          # mssSorIt
    sortol: float = 1.0e-8      # ssSorTol
    sorrel: float = 1.0         # ssSorRel
    cu0: float = 0.0            # ssCu0
    tscoef: float = 1.0         # ssTsCoef
    hscoef: float = 1.0         # ssHsCoef
    temcoef: float = 1.0        # ssTemCoef
    bnumc: float = 200.0        # ssBnCrit
    rmax: float = 0.95          # ssRMpMax
    rlc: float = 5.0            # ssRMpExp
    fpu: float = 500.0          # ssFiltPar(_U_)
    fpv: float = 500.0          # ssFiltPar(_V_)
    fpt: float = 500.0          # ssFiltPar(_T_)
    dlref: float = 1.0
    uref: float = 1.0
    tref: float = 300.0
    tmax: float = 330.0
    pe: float = 0.0             # re * Prandtl


@dataclasses.dataclass
class ThermalParams:
    """Thermal switches and constants of the time loop: ReadParam's
    nthermen, neqstate, nmeiter, dmeittol (defaults src/parse.f:118-159),
    pe = re * Prandtl (src/file_manip.f:158) and EqState's constants."""
    nthermen: int = 1
    neqstate: int = 0
    nmeiter: int = 1
    dmeittol: float = 1.0e-4
    pe: float = 1.0
    uref: float = 1.0
    densref: float = 1.0
    tmax: float = 1.0
    tref: float = 0.0
    rconst: float = 1.0
    nfiltt: int = 0             # Filter of t after the iterations (filter_t)
    fpt: float = 5.0            # its parameter (src/parse.f:159 default)


@dataclasses.dataclass
class Case:
    """Everything the hot path needs for one instance."""
    name: str
    nx: int
    ny: int
    x: np.ndarray   # node x coordinates, shape (nx, ny), already / dlref
    y: np.ndarray
    regions: Regions
    params: RunParams
    bc_text: str = ""
    thermal: Optional[Thermal] = None        # thermal tables (nthermen = 1)
    tparams: Optional[ThermalParams] = None
    atd: Optional[SmallScaleParams] = None   # nsmallscl = 1 (needs the thermal tables)

    @property
    def cells(self) -> int:
        return (self.nx - 1) * (self.ny - 1)


def _uniform_nodes(ncx: int, ncy: int, lx: float, ly: float):
    xi = np.array([lx * i / ncx for i in range(ncx + 1)], np.float64)
    yj = np.array([ly * j / ncy for j in range(ncy + 1)], np.float64)
    X = np.repeat(xi[:, None], ncy + 1, axis=1)
    Y = np.repeat(yj[None, :], ncx + 1, axis=0)
    return X, Y


def cavity(n: int, re: float, dt: float, *, lid: float = 1.0,
           solver: str = "sor", ny: Optional[int] = None, side: float = 1.0, **kw) -> Case:
    """Lid-driven cavity of width ``side`` (the unit square by default) with
    n x n uniform cells: no-slip walls, north wall moving at ``lid`` (``wall
    1 1 north tv <lid>``), fluid with rho = 1 and mu = 1/re, dlref = uref = 1."""
    ncy = n if ny is None else ny
    X, Y = _uniform_nodes(n, ncy, side, side * float(ncy) / n)
    nx, nyy = n + 1, ncy + 1
    bc = ("number_of_regions 1 1\n"
          "i_borders\n"
          "j_borders\n"
          f"wall 1 1 north tv {lid!r}\n")
    prm = RunParams.scaled(dt, 1.0, 1.0, 1.0, 1.0 / re,
                           npsolver=PPE_SOLVERS[solver], lcartes=1, **kw)
    regs = parse_bc_section(bc, nx, nyy, re=prm.re)
    return Case(f"cavity{n}x{ncy}_re{re:g}", nx, nyy, X, Y, regs, prm, bc)


def clustered_cavity(n: int, re: float, dt: float, *, beta: float = 0.5, **kw) -> Case:
    """The lid-driven cavity of ``cavity`` on a Cartesian grid whose cells
    cluster towards the walls: node k of either direction at
    s - beta sin(2 pi s) / (2 pi), s = k / n, so cell widths run from (1 -
    beta) / n at the walls to (1 + beta) / n in the middle and no Poisson
    row is the unit stencil."""
    case = cavity(n, re, dt, **kw)
    warp = lambda s: s - beta * np.sin(2.0 * np.pi * s) / (2.0 * np.pi)
    case.x = np.asfortranarray(warp(case.x))
    case.y = np.asfortranarray(warp(case.y))
    case.name = f"clustered{n}_re{re:g}"
    return case


def heated_cavity(n: int, re: float, dt: float, *, pr: float = 0.71, fr: float = 0.05,
                  lid: float = 0.0, nmeiter: int = 3, dmeittol: float = 1.0e-6,
                  eqstate: bool = True, solver: str = "rb_sor", t_hot: float = 1.0,
                  t_cold: float = 0.0, **kw) -> Case:
    """Differentially heated cavity: the cavity of :func:`cavity` (moving
    lid optional) with the energy equation on (nthermen = 1, pe = re * pr):
    west wall at t_hot, east wall at t_cold (fixed temperature), adiabatic
    south and north walls (zero heat flux); with ``eqstate`` the density of
    the ideal-gas EqState (tref = 300, tmax = 330, so d ~ -0.1 t) drives the
    buoyancy term of YMomentum at Froude number ``fr``."""
    case = cavity(n, re, dt, lid=lid, solver=solver, **kw)
    case.params.fr = fr
    th = Thermal.empty()
    th.nTemBdTp[0, 0, :] = (BT_TEMPER, BT_TEMPER, BT_HTFLUX, BT_HTFLUX)
    case.regions.dBCVal[0, 0, WEST - 1, VAR_T - 1] = t_hot
    case.regions.dBCVal[0, 0, EAST - 1, VAR_T - 1] = t_cold
    case.thermal = th
    case.tparams = ThermalParams(nthermen=1, neqstate=1 if eqstate else 0, nmeiter=nmeiter,
                                 dmeittol=dmeittol, pe=case.params.re * pr, uref=1.0, densref=1.0,
                                 tmax=330.0, tref=300.0, rconst=287.0)
    case.name = f"heated_{case.name}"
    return case


def channel(ncx: int, ncy: int, re: float, dt: float, *, length: float = 4.0,
            height: float = 1.0, u_in: float = 1.0, solver: str = "rb_sor",
            outlet: str = "fd", **kw) -> Case:
    """Plane channel: inlet on the west face with normal velocity ``u_in``,
    outlet on the east face (``fd`` fully developed, bound_cond.f BM_OUTLT1;
    ``mc`` mass conservation, BM_OUTLT2), no-slip south/north walls."""
    X, Y = _uniform_nodes(ncx, ncy, length, height)
    nx, ny = ncx + 1, ncy + 1
    bc = ("number_of_regions 1 1\n"
          "i_borders\n"
          "j_borders\n"
          f"inlet 1 1 west nv {u_in!r}\n"
          f"outlet 1 1 east {outlet}\n")
    prm = RunParams.scaled(dt, 1.0, 1.0, 1.0, 1.0 / re,
                           npsolver=PPE_SOLVERS[solver], lcartes=1, **kw)
    regs = parse_bc_section(bc, nx, ny, re=prm.re)
    return Case(f"channel{ncx}x{ncy}_re{re:g}", nx, ny, X, Y, regs, prm, bc)


def inflow_profile(case: Case, seed: int, amp: float = 1.0e-2, modes: int = 16,
                   u_center: float = 1.0) -> np.ndarray:
    """Parabolic inflow plus a seeded Fourier perturbation, as the u values
    of the west face over j = 0..ny+1: at row j (between nodes j-1 and j)
    with centre height y_c, u = 4 u_center y_c (H - y_c) / H^2 + sum_k a_k
    sin(k pi y_c / H), a_k ~ N(0, amp^2) from default_rng(seed), k = 1..modes;
    0 on the rows outside the channel."""
    y = case.y[0, :]
    y0, h_ch = y[0], y[-1] - y[0]
    rng = np.random.default_rng(seed)
    a = rng.normal(0.0, amp, size=modes)
    prof = np.zeros(case.ny + 2)
    for j in range(2, case.ny + 1):
        yc = 0.5 * (y[j - 2] + y[j - 1]) - y0
        s = 4.0 * u_center * yc * (h_ch - yc) / h_ch ** 2
        s += float(np.dot(a, np.sin(np.arange(1, modes + 1) * np.pi * yc / h_ch)))
        prof[j] = s
    return prof


def channel_inflow(ncx: int, ncy: int, re: float, dt: float, *, seed: int = 1234,
                   length: float = 4.0, height: float = 1.0, amp: float = 1.0e-2,
                   solver: str = "rb_sor", outlet: str = "mc", **kw) -> Case:
    """Plane channel with a parabolic + perturbed inflow profile on the west
    face (a per-row face profile: the reference's faces carry one constant),
    outlet on the east face, no-slip walls.

    The default outlet is the mass-conserving one (bound_cond.f BM_OUTLT2:
    zero-gradient u corrected by continuity, u(iE) = u(iE-1) - (v(iE,j) -
    v(iE,j-1))).  With the fully developed outlet (``fd``, BM_OUTLT1) the
    outflow does not balance the inflow, the all-Neumann pressure problem has
    no solution, and the scheme grows without bound within a few steps."""
    case = channel(ncx, ncy, re, dt, length=length, height=height, u_in=1.0, solver=solver,
                   outlet=outlet, **kw)
    case.regions.profiles[(1, 1, WEST, 1)] = inflow_profile(case, seed, amp)
    case.name = f"channel{ncx}x{ncy}_re{re:g}_profiled"
    return case


def channel_ic(case: Case):
    """Initial fields of a profiled channel: u = the inflow profile in every
    column (divergence-free: u depends on j only, v = 0), p = 0."""
    prof = case.regions.profiles[(1, 1, WEST, 1)]
    u = np.zeros((case.nx + 2, case.ny + 2), order="F")
    u[:, :] = prof[None, :]
    return u, np.zeros_like(u), np.zeros_like(u)


ENSEMBLE_SIZES = tuple(range(64, 513, 32))


@dataclasses.dataclass
class EnsembleMember:
    case: Case
    n: int           # cells per side
    re: float        # cavity Reynolds number U L / nu
    dt_named: float  # 0.5 h
    dt: float        # the step used


def ensemble_cases(count: int = 256, seed: int = 2024, visc_max: float = 0.25,
                   solver: str = "rb_sor") -> List[EnsembleMember]:
    """The batched-ensemble workload: ``count`` lid-driven cavities on the
    unit square, N cells per side drawn uniformly from {64, 96, ..., 512}
    and the cavity Reynolds number log-uniform in [100, 5000], both from
    default_rng(seed), h = 1/N, dt = 0.5 h.

    The reference's scheme is unstable above a viscous number dt/(h^2 Re)
    of about 0.3 (0.64 reaches NaN within 8 steps), and 0.5 h / (h^2 Re) =
    0.5 N / Re exceeds that for small Re and large N, so dt is capped at
    visc_max h^2 Re; ``dt_named`` and ``dt`` record both."""
    rng = np.random.default_rng(seed)
    ns = rng.choice(np.array(ENSEMBLE_SIZES), size=count)
    res = np.exp(rng.uniform(np.log(100.0), np.log(5000.0), size=count))
    out = []
    for n, re in zip(ns.tolist(), res.tolist()):
        h = 1.0 / n
        dt_named = 0.5 * h
        dt = min(dt_named, visc_max * h * h * re)
        case = cavity(n, re, dt, solver=solver)
        case.name = f"ens_cavity{n}_re{re:.1f}"
        out.append(EnsembleMember(case, n, re, dt_named, dt))
    return out


def perturbation_ic(case: Case, seed: int, modes: int = 16, amp: float = 1.0e-3):
    """Seeded divergence-free initial velocity on the staggered grid.

    psi(x,y) = sum_{k,l=1..modes} a_kl sin(k pi x/Lx) sin(l pi y/Ly) with
    a_kl ~ N(0, amp^2) from numpy.random.default_rng(seed); then
    u(i,j) = (psi(i,j) - psi(i,j-1))/hy and v(i,j) = -(psi(i,j) - psi(i-1,j))/hx
    at the staggered u/v locations, so the discrete divergence (pressure.f
    nloc = 1) vanishes up to rounding and the walls see zero normal flow.
    Returns (u, v, p) as Fortran-ordered (nx+2, ny+2) arrays; p = 0."""
    rng = np.random.default_rng(seed)
    a = rng.normal(0.0, amp, size=(modes, modes))
    x = case.x[:, 0]
    y = case.y[0, :]
    lx, ly = x[-1] - x[0], y[-1] - y[0]
    k = np.arange(1, modes + 1)
    sx = np.sin(np.pi * np.outer(x - x[0], k) / lx)     # (nx, modes)
    sy = np.sin(np.pi * np.outer(y - y[0], k) / ly)     # (ny, modes)
    psi = sx @ a @ sy.T                                  # (nx, ny)
    nx, ny = case.nx, case.ny
    hx = np.diff(x)
    hy = np.diff(y)
    u = np.zeros((nx + 2, ny + 2), order="F")
    v = np.zeros((nx + 2, ny + 2), order="F")
    u[1:nx + 1, 2:ny + 1] = (psi[:, 1:] - psi[:, :-1]) / hy[None, :]
    v[2:nx + 1, 1:ny + 1] = -(psi[1:, :] - psi[:-1, :]) / hx[:, None]
    p = np.zeros((nx + 2, ny + 2), order="F")
    return u, v, p


# ---------------------------------------------------------------------------
# Reference-format files: decks, Plot3D grid, fluid table, restart records.
# ---------------------------------------------------------------------------

def write_grid_plot3d(path: str, x: np.ndarray, y: np.ndarray) -> None:
    """2-D formatted Plot3D grid read by ReadGrid (src/grid.f:189-228):
    first line ``nx ny``, then all x (i fastest), then all y."""
    nx, ny = x.shape
    with open(path, "w") as f:
        f.write(f"{nx} {ny}\n")
        for arr in (x, y):
            vals = arr.ravel(order="F")
            for k in range(0, vals.size, 4):
                f.write(" ".join(repr(float(v)) for v in vals[k:k + 4]) + "\n")


def write_deck(path: str, case: Case, *, grid_file: str = "grid.xyz",
               nts: int = 1, print_diff: int = 1) -> None:
    """Input deck with the two sections the reference reads from one file
    (src/main.f:311-312)."""
    inv = {v: k for k, v in PPE_SOLVERS.items()}
    p = case.params
    with open(path, "w") as f:
        f.write("section input_parameters\n")
        f.write(f"  grid_file {grid_file}{' cartesian_grid' if p.lcartes else ''}\n")
        f.write(f"  n_time_steps {nts}\n")
        f.write(f"  time_step_size {p.dk!r}\n")
        f.write(f"  max_ql_iter {p.mqiter}\n  ql_tolerance {p.qtol!r}\n")
        f.write(f"  ppe_solver {inv[p.npsolver]}\n")
        f.write(f"  max_sor_iter {p.msorit}\n  sor_tolerance {p.sortol!r}\n")
        f.write(f"  sor_relaxation {p.sorrel!r}\n")
        f.write(f"  print_diff_freq {print_diff}\n")
        f.write("end section\n\n")
        f.write("section boundary_conditions\n")
        for line in case.bc_text.splitlines():
            f.write("  " + line + "\n")
        f.write("end section\n")


def write_fluid_table(path: str, rho: float, mu: float, name: str = "air01") -> None:
    """Fluid table with two identical rows at T = 200 and 400 so the
    interpolation at tref returns them exactly (src/utility.f:654-662)."""
    with open(path, "w") as f:
        f.write(f"fluid {name}\n")
        for temp in (200.0, 400.0):
            f.write(f"{temp!r} {rho!r} 1.0 {mu!r} 1.0 1.0\n")
        f.write("end\n")


def write_restart(path: str, k: int, dtime: float, nx: int, ny: int,
                  fields: Sequence[np.ndarray]) -> None:
    """Fortran unformatted sequential restart file (src/file_manip.f:364-401):
    record 1 ``k, dtime``; record 2 ``nx, ny``; record 3 the eight fields
    p, u, v, t, pss, uss, vss, tss over (0:nx+1, 0:ny+1).  Each record is
    framed by 4-byte little-endian length markers (gfortran)."""
    def rec(buf: bytes) -> bytes:
        n = np.array([len(buf)], "<i4").tobytes()
        return n + buf + n
    body = [rec(np.array([k], "<i4").tobytes() + np.array([dtime], "<f8").tobytes()),
            rec(np.array([nx, ny], "<i4").tobytes())]
    parts = []
    for fld in fields:
        parts.append(np.asarray(fld[: nx + 2, : ny + 2], "<f8").ravel(order="F").tobytes())
    body.append(rec(b"".join(parts)))
    with open(path, "wb") as f:
        f.write(b"".join(body))


def write_plot3d_solution(prefix: str, nx: int, ny: int, u: np.ndarray, v: np.ndarray,
                          p: np.ndarray, t: Optional[np.ndarray] = None,
                          names: bool = True) -> None:
    """The standard-variable output of SaveStdVarsP3D (src/file_manip.f:1024-1175)
    in its unformatted form: ``<prefix>.qqq`` holds record 1 ``nx, ny, nVars``
    and record 2 the REAL*8 functions f(i, j, l) over i = 1..nx, j = 1..ny
    (i fastest) for l = p, u, v, w = 0 (and t with the energy equation);
    ``<prefix>.nam`` the FieldView names, one list-directed line each."""
    def rec(buf: bytes) -> bytes:
        n = np.array([len(buf)], "<i4").tobytes()
        return n + buf + n
    funcs = [p, u, v, np.zeros_like(p)] + ([t] if t is not None else [])
    body = rec(np.array([nx, ny, len(funcs)], "<i4").tobytes())
    data = b"".join(np.asarray(f[1:nx + 1, 1:ny + 1], "<f8").ravel(order="F").tobytes() for f in funcs)
    with open(prefix + ".qqq", "wb") as fh:
        fh.write(body + rec(data))
    if names:
        lines = ["Complete Pressure", "Complete U ; Complete Velocity", "Complete V", "Complete W"]
        if t is not None:
            lines.append("Complete Temperature")
        with open(prefix + ".nam", "w") as fh:
            fh.write("".join(f" {x}\n" for x in lines))


def read_plot3d_solution(path: str):
    """Inverse of :func:`write_plot3d_solution` for the .qqq file: returns
    (nx, ny, f) with f of shape (nx, ny, nVars)."""
    b = open(path, "rb").read()
    n0 = int(np.frombuffer(b[:4], "<i4")[0])
    nx, ny, nv = (int(x) for x in np.frombuffer(b[4:4 + n0], "<i4"))
    o = 4 + n0 + 4
    n1 = int(np.frombuffer(b[o:o + 4], "<i4")[0])
    f = np.frombuffer(b[o + 4:o + 4 + n1], "<f8").reshape((nx, ny, nv), order="F")
    return nx, ny, f


def read_restart(path: str):
    """Inverse of :func:`write_restart`; returns (k, dtime, nx, ny, fields)."""
    data = open(path, "rb").read()
    pos = 0
    recs = []
    while pos < len(data):
        n = int(np.frombuffer(data, "<i4", 1, pos)[0])
        recs.append(data[pos + 4: pos + 4 + n])
        pos += 8 + n
    k = int(np.frombuffer(recs[0], "<i4", 1, 0)[0])
    dtime = float(np.frombuffer(recs[0], "<f8", 1, 4)[0])
    nx, ny = (int(v) for v in np.frombuffer(recs[1], "<i4", 2, 0))
    arr = np.frombuffer(recs[2], "<f8").reshape(8, ny + 2, nx + 2)
    fields = [np.asfortranarray(a.T) for a in arr]
    return k, dtime, nx, ny, fields


# ---- input_parameters section and fluid table (ReadParam) -----------------

@dataclasses.dataclass
class DeckInput:
    """The input_parameters section as ReadParam leaves it (src/parse.f:117-193
    defaults, src/parse.f:261-903 keywords), before the reference scaling."""
    grid_file: str = ""
    lcartes: int = 0
    nthermen: int = 0
    neqstate: int = 0
    nts: int = 0
    dt: float = 0.0                 # physical time step (time_step_size)
    mqiter: int = 20
    qtol: float = 1.0e-4
    nmeiter: int = 1
    dmeittol: float = 1.0e-4
    nfiltu: int = 0
    nfiltv: int = 0
    nfiltt: int = 0
    fpu: float = 5.0e2
    fpv: float = 5.0e2
    fpt: float = 5.0
    npsolver: int = 1
    msorit: int = 2000
    sortol: float = 1.0e-8
    sorrel: float = 1.0
    dlref: float = 1.0
    uref: float = 1.0
    tref: float = 283.57
    tmax: float = 1.0e3
    fluid_file: str = "fluidprop.dat"
    fluid_name: str = "air01"
    restart: Optional[str] = None
    write_restart: Optional[str] = None
    write_restart_freq: int = 0     # 0: at the end only
    print_diff_freq: int = 1
    other: dict = dataclasses.field(default_factory=dict)  # keywords off the hot path, as read


_INT_KEYS = {"n_time_steps": "nts", "max_ql_iter": "mqiter", "max_me_iter": "nmeiter",
             "max_sor_iter": "msorit", "print_diff_freq": "print_diff_freq"}
_REAL_KEYS = {"time_step_size": "dt", "ql_tolerance": "qtol", "me_tolerance": "dmeittol",
              "sor_tolerance": "sortol", "sor_relaxation": "sorrel", "ref_length": "dlref",
              "ref_velocity": "uref", "ref_temperature": "tref", "max_ref_temperature": "tmax"}
_FILTER_KEYS = {"filter_u": ("nfiltu", "fpu"), "filter_v": ("nfiltv", "fpv"), "filter_t": ("nfiltt", "fpt")}
# accepted and kept as read: ATD, time averaging, trajectories and output control
_OTHER_KEYS = {"small_scale", "trajectories", "atd_cu0", "atd_tscf", "atd_hscf", "atd_bnumcrit",
               "atd_rmapmax", "atd_rmapexp", "atd_temcf", "atd_ppe_solver", "atd_max_sor_iter",
               "atd_sor_tolerance", "atd_sor_relaxation", "atd_filter_u", "atd_filter_v", "atd_filter_t",
               "time_average_mode", "output_format", "output_prefix", "snapshots_prefix", "snapshots_freq",
               "snapshots_first", "time_series_prefix", "time_series_freq", "time_series_point",
               "print_bann_freq"}


def _sections(text: str):
    """{section name: body text} of a deck (``section <name>`` ... ``end
    section``, case-insensitive keywords, ``#`` comments)."""
    out, cur, body = {}, None, []
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].strip()
        w = line.lower().split()
        if not w:
            continue
        if w[0] == "section":
            if cur is not None or len(w) < 2:
                raise DeckError("SECTION keyword misplaced")
            cur, body = w[1], []
        elif w[0] == "end" and len(w) > 1 and w[1] == "section":
            if cur is None:
                raise DeckError("END SECTION without SECTION")
            out[cur] = "\n".join(body)
            cur = None
        elif cur is not None:
            body.append(line)
    if cur is not None:
        raise DeckError(f"section {cur} not closed")
    return out


def parse_input_section(text: str) -> DeckInput:
    """The input_parameters keywords (src/parse.f:261-903)."""
    d = DeckInput()
    for raw in text.splitlines():
        w = raw.split("#", 1)[0].split()
        if not w:
            continue
        key = w[0].lower()

        def arg(k=1):
            if len(w) <= k:
                raise DeckError(f"{key}: value missing")
            return w[k]
        try:
            if key == "grid_file":
                d.grid_file = arg()
                if len(w) > 2:
                    if w[2].lower() != "cartesian_grid":
                        raise DeckError(f"Unrecognized keyword: [{w[2]}]")
                    d.lcartes = 1
            elif key == "thermal_energy":
                d.nthermen = 1
            elif key == "buoyancy":
                d.neqstate = 1
            elif key in _INT_KEYS:
                setattr(d, _INT_KEYS[key], int(arg()))
            elif key in _REAL_KEYS:
                setattr(d, _REAL_KEYS[key], float(arg().replace("d", "e").replace("D", "e")))
            elif key in _FILTER_KEYS:
                flag, par = _FILTER_KEYS[key]
                setattr(d, flag, 1)
                setattr(d, par, float(arg().replace("d", "e").replace("D", "e")))
            elif key == "ppe_solver":
                name = arg().lower()
                if name not in PPE_SOLVERS:
                    raise DeckError(f"Unrecognized ppe_solver: [{name}]")
                d.npsolver = PPE_SOLVERS[name]
            elif key == "fluid_prop_file":
                d.fluid_file = arg()
            elif key == "fluid_prop_table":
                d.fluid_name = arg()
            elif key == "restart":
                d.restart = arg()
            elif key == "write_restart":
                d.write_restart = arg()
                d.write_restart_freq = int(w[2]) if len(w) > 2 else 0
            elif key in _OTHER_KEYS:
                d.other[key] = w[1:]
            else:
                raise DeckError(f"Unrecognized keyword: [{key}]")
        except ValueError as exc:
            raise DeckError(f"{key}: bad value {' '.join(w[1:])!r}") from exc
    return d


def read_fluid_props(path: str, name: str, tref: float) -> dict:
    """lReadFldProps (src/parse.f:2027-2250): the rows ``T rho c mu k Pr`` of
    fluid ``name`` (optional ``gasconstant R`` on its ``fluid`` line), linearly
    interpolated at tref between the bracketing rows as dLinInterp does
    (src/utility.f:654-662: y1 + (y2 - y1)(x - x1)/(x2 - x1), with the
    current row as point 1 and the previous one as point 2)."""
    found, inside, prev, rconst = False, False, None, 0.0
    nrow = 0
    for raw in open(path):
        line = raw.strip()
        if not line:
            continue
        if line.startswith("#"):
            if inside:
                raise DeckError("Comments not allowed inside Fluid Def.")
            continue
        w = line.lower().split()
        if w[0] == "fluid" and not inside:
            inside, nrow, prev = True, 0, None
            found = len(w) > 1 and w[1] == name.lower()
            if found and len(w) > 3 and w[2] == "gasconstant":
                rconst = float(w[3])
            continue
        if w[0] == "end" and inside:
            inside = False
            if found:
                raise DeckError("Did not find requested interval")
            continue
        if inside and found:
            nrow += 1
            row = [float(x) for x in w[:6]]
            if nrow == 1 and row[0] > tref:
                raise DeckError(f"Searched value ({tref}) is lower than first entry in table")
            p = prev if prev is not None else [0.0] * 6
            if nrow > 1 and p[0] > row[0]:
                raise DeckError("Entries should be arranged in ascending order with respect to temperature")
            if p[0] <= tref <= row[0]:
                vals = [row[k] + (p[k] - row[k]) * (tref - row[0]) / (p[0] - row[0]) for k in range(1, 6)]
                return {"tref": tref, "densref": vals[0], "c": vals[1], "mu": vals[2],
                        "dconduct": vals[3], "prandtl": vals[4], "rconst": rconst}
            prev = row
    raise DeckError(f"fluid {name!r} not found in {path}")


def read_grid_plot3d(path: str):
    """2-D formatted Plot3D grid as ReadGrid reads it (src/grid.f:189-228):
    ``nx ny``, then every x (i fastest), then every y; returns (nx, ny, X, Y)
    with X, Y of shape (nx, ny)."""
    vals = open(path).read().replace("d", "e").replace("D", "e").split()
    nx, ny = int(vals[0]), int(vals[1])
    a = np.array([float(v) for v in vals[2:2 + 2 * nx * ny]])
    X = a[:nx * ny].reshape((nx, ny), order="F")
    Y = a[nx * ny:].reshape((nx, ny), order="F")
    return nx, ny, X, Y


def read_deck(path: str, base: Optional[str] = None) -> Case:
    """A reference input deck (both sections, src/main.f:311-312) with its grid
    and fluid files (relative to ``base``, default the deck's folder) as a
    Case: ReadParam's scaling (src/file_manip.f:130-157: dk = dt uref/dlref,
    Re = dlref uref rho/mu, Pe = Re Pr, Fr = uref^2/(9.81 dlref)), the grid
    nodes divided by dlref, the boundary section with its thermal tables, and
    the heat sources of bound_cond.f:2018-2029."""
    import os
    base = base if base is not None else os.path.dirname(os.path.abspath(path))
    sec = _sections(open(path).read())
    if "input_parameters" not in sec or "boundary_conditions" not in sec:
        raise DeckError("a deck needs input_parameters and boundary_conditions sections")
    d = parse_input_section(sec["input_parameters"])
    fl = read_fluid_props(os.path.join(base, d.fluid_file), d.fluid_name, d.tref)
    kinvisc = fl["mu"] / fl["densref"]
    re = d.dlref * d.uref / kinvisc
    fr = d.uref ** 2.0 / (d.dlref * 9.81)
    prm = RunParams(dk=d.dt * d.uref / d.dlref, re=re, fr=fr, nts=d.nts, mqiter=d.mqiter, qtol=d.qtol,
                    npsolver=d.npsolver, msorit=d.msorit, sortol=d.sortol, sorrel=d.sorrel,
                    nfiltu=d.nfiltu, nfiltv=d.nfiltv, fpu=d.fpu, fpv=d.fpv, lcartes=d.lcartes)
    nx, ny, X, Y = read_grid_plot3d(os.path.join(base, d.grid_file))
    regs = parse_bc_section(sec["boundary_conditions"], nx, ny, uref=d.uref, densref=fl["densref"],
                            dlref=d.dlref, re=re, tref=fl["tref"], tmax=d.tmax)
    case = Case(os.path.splitext(os.path.basename(path))[0], nx, ny, X / d.dlref, Y / d.dlref, regs, prm,
                sec["boundary_conditions"])
    if d.nthermen or d.neqstate:
        pe = re * fl["prandtl"]
        if d.nthermen:
            heat_sources(regs, d.dlref, fl["tref"], d.tmax, fl["dconduct"], pe)
        case.thermal = regs.thermal
        case.tparams = ThermalParams(nthermen=d.nthermen, neqstate=d.neqstate, nmeiter=d.nmeiter,
                                     dmeittol=d.dmeittol, pe=pe, uref=d.uref, densref=fl["densref"],
                                     tmax=d.tmax, tref=fl["tref"], rconst=fl["rconst"], nfiltt=d.nfiltt,
                                     fpt=d.fpt)
    if "small_scale" in d.other:
        case.thermal = case.thermal if case.thermal is not None else regs.thermal
        case.atd = small_scale_params(d, pe=re * fl["prandtl"], tref=fl["tref"])
    return case


_ATD_REAL = {"atd_cu0": "cu0", "atd_tscf": "tscoef", "atd_hscf": "hscoef", "atd_bnumcrit": "bnumc",
             "atd_rmapmax": "rmax", "atd_rmapexp": "rlc", "atd_temcf": "temcoef",
             "atd_sor_tolerance": "sortol", "atd_sor_relaxation": "sorrel", "atd_filter_u": "fpu",
             "atd_filter_v": "fpv", "atd_filter_t": "fpt"}


def small_scale_params(d: DeckInput, pe: float, tref: float) -> SmallScaleParams:
    """SmallScale's parameters from the atd_* keywords of a deck (src/parse.f:
    491-620, defaults 144-178) and the deck's reference scales."""
    a = SmallScaleParams(dlref=d.dlref, uref=d.uref, tref=tref, tmax=d.tmax, pe=pe)
    for key, w in d.other.items():
        try:
            if key in _ATD_REAL:
                setattr(a, _ATD_REAL[key], float(w[0].replace("d", "e").replace("D", "e")))
            elif key == "atd_max_sor_iter":
                a.msorit = int(w[0])
            elif key == "atd_ppe_solver":
                if w[0].lower() not in PPE_SOLVERS:
                    raise DeckError(f"Unrecognized atd_ppe_solver: [{w[0]}]")
                a.npsolver = PPE_SOLVERS[w[0].lower()]
        except (IndexError, ValueError) as exc:
            raise DeckError(f"{key}: bad value {' '.join(w)!r}") from exc
    return a
