"""A thermal test problem for ThermEnergy / TempBoundCond / EqState: a 3 x 2
region layout on a curvilinear grid (so every metric term of the thermal
right-hand side is non-zero), one fixed-temperature region, one
heat-generating region, fixed-temperature and heat-flux outer faces and
seeded smooth fields."""
import numpy as np

from wolfd2_gb300 import deck
from wolfd2_gb300.deck import (BT_HTFLUX, BT_INTERN, BT_TEMPER, EAST, NORTH, RT_HEATGN, RT_TEMPER,
                               SOUTH, VAR_T, WEST)


def problem(ncx: int = 36, ncy: int = 24, seed: int = 5):
    text = ("number_of_regions 3 2\n i_borders 13 25\n j_borders 11\n"
            "wall 1 1 south\n wall 2 1 south\n wall 3 1 south\n"
            "wall 1 2 north tv 1.0\n wall 2 2 north tv 1.0\n wall 3 2 north tv 1.0\n")
    case = deck.cavity(ncx, 200.0, 0.004, solver="rb_sor", ny=ncy)
    case.regions = deck.parse_bc_section(text, case.nx, case.ny, re=case.params.re)
    case.bc_text = text
    rng = np.random.default_rng(seed)
    # curvilinear nodes: a smooth displacement that keeps the boundary lines
    # straight at the four edges
    X, Y = case.x.copy(), case.y.copy()
    sx = np.sin(np.pi * X) * np.sin(np.pi * Y)
    case.x = X + 0.02 * sx
    case.y = Y + 0.015 * np.sin(2 * np.pi * X) * np.sin(np.pi * Y)
    th = deck.Thermal.empty()
    th.nTRgType[1, 0] = RT_TEMPER
    th.dTRgVal[1, 0] = 0.7
    th.nTRgType[0, 1] = RT_HEATGN
    th.dHGSTval[0, 1] = 0.3
    nri, nrj = 3, 2
    for ir in range(nri):
        for jr in range(nrj):
            for face in (WEST, EAST, SOUTH, NORTH):
                outer = ((face == WEST and ir == 0) or (face == EAST and ir == nri - 1) or
                         (face == SOUTH and jr == 0) or (face == NORTH and jr == nrj - 1))
                if outer:
                    bt = BT_TEMPER if face in (WEST, SOUTH) else BT_HTFLUX
                else:
                    bt = BT_INTERN
                th.nTemBdTp[ir, jr, face - 1] = bt
                case.regions.dBCVal[ir, jr, face - 1, VAR_T - 1] = rng.uniform(-0.5, 1.0)
    # faces of the fixed-temperature region's neighbours are fixed-temperature
    th.nTemBdTp[0, 0, EAST - 1] = BT_TEMPER
    th.nTemBdTp[2, 0, WEST - 1] = BT_TEMPER
    th.nTemBdTp[1, 1, SOUTH - 1] = BT_TEMPER
    mnx, mny = case.nx + 1, case.ny + 1
    ii, jj = np.meshgrid(np.arange(mnx + 1), np.arange(mny + 1), indexing="ij")

    def smooth(k):
        a = rng.normal(size=(3, 3))
        f = sum(a[p, q] * np.sin((p + 1) * np.pi * ii / mnx + k) * np.cos((q + 1) * np.pi * jj / mny)
                for p in range(3) for q in range(3))
        return np.asfortranarray(f)
    fields = {n: smooth(k) for k, n in enumerate(["u", "v", "un", "vn", "tn", "t", "p"])}
    fields["t"] = np.asfortranarray(fields["tn"] + 0.01 * fields["t"])
    return case, th, fields


def loop_case(nmeiter: int = 3):
    """The 3 x 2 thermal layout as a time-loop case: energy equation and
    EqState on (buoyancy at Froude number 0.05), momentum/energy iterations."""
    case, th, f = problem()
    case.thermal = th
    case.tparams = deck.ThermalParams(nthermen=1, neqstate=1, nmeiter=nmeiter, dmeittol=1e-7, pe=100.0,
                                      tmax=330.0, tref=300.0, rconst=287.0)
    case.params.fr = 0.05
    return case


def curvilinear_case(lcartes: int = 0):
    """The 3 x 2 curvilinear layout without the energy equation, for the
    plain time loop on a non-Cartesian grid (RhsPpe's cross terms every
    sweep when lcartes = 0)."""
    case, th, f = problem()
    case.params.lcartes = lcartes
    return case


def blockage_case():
    """Three regions in i with an internal blockage, an inlet and an outlet."""
    text = ("number_of_regions 3 1\n i_borders 12 20\n j_borders\n"
            "blockage 2 1\n inlet 1 1 west nv 1.0\n outlet 3 1 east fd\n")
    case = deck.channel(32, 14, 300.0, 0.003, length=2.0, solver="rb_sor")
    case.regions = deck.parse_bc_section(text, case.nx, case.ny, re=case.params.re)
    case.bc_text = text
    return case
