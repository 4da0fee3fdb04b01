"""SmallScale (small_scale.f:31-578) with SmlSclBC (bound_cond.f:1211-1500)
on the device, through the C-ABI, against the oracle's restatement (itself
pinned bit for bit to the translated reference source).

The device evaluates the reference's expressions in its operand order, but
pow, tanh and atanh are CUDA's, an ulp or so from the host's, and the
logistic maps are chaotic for rmap near rmax.  So the bar depends on the
maps: with cu0 = 0 (parse.f's default: no map is iterated) every field is
bit-identical over four calls; with maps that contract (bnumc = 200, rmap
about 1e-6) the small scales agree to 1e-11 of their size; with chaotic maps
(bnumc = 5) a cell's values are not reproducible after tens of iterations
on either machine, and the test compares what the maps do not decide: the
cells the model acts on, the pressure sweep counts, and the size of the
small scales."""
import os
import sys

import numpy as np
import pytest

import oracle as O
from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import Solver

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def _layout(name):
    import thermal_setup
    if name == "blockage":
        case = thermal_setup.blockage_case()
        th = deck.Thermal.empty()
        rng = np.random.default_rng(3)
        u, v, p = deck.perturbation_ic(case, 5, amp=0.3)
        t = np.asfortranarray(rng.uniform(0.0, 1.0, size=u.shape))
        return case, th, u, v, t
    case, th, f = thermal_setup.problem()
    case.params.lcartes = 0
    t = np.asfortranarray(0.5 + 0.4 * np.tanh(f["tn"]))
    return case, th, np.asfortranarray(f["u"]), np.asfortranarray(f["v"]), t


def _run(layout, cu0, bnumc, dka, calls=4):
    case, th, u, v, t = _layout(layout)
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    ap = O.AtdParams.make(dka=dka, re=1000.0, pe=700.0, npsolver=deck.PPE_SOLVERS["rb_sor"], msorit=300,
                          lcartes=case.params.lcartes, cu0=cu0, sortol=1e-9, sorrel=1.2,
                          fp=(400.0, 300.0, 0.0, 200.0), bnumc=bnumc)
    atd = O.SmallScale(o, case.nx, case.ny, case.regions, th, met, ap)
    s = Solver.for_case(case, tuned=False)
    orc = {k: o.field() for k in ("uss", "vss", "pss", "tss")}
    dev = {k: o.field() for k in ("uss", "vss", "pss", "tss")}
    rng = np.random.default_rng(11)
    out = []
    for call in range(calls):
        flg = 0 if call == 0 else 1
        n_o = atd(flg, u, v, t, orc["uss"], orc["vss"], orc["pss"], orc["tss"])
        n_d = s.SmallScale(flg, th, ap, u, v, t, dev["uss"], dev["vss"], dev["pss"], dev["tss"])
        out.append((n_o, n_d, {k: w.copy() for k, w in orc.items()}, {k: w.copy() for k, w in dev.items()}))
        u = np.asfortranarray(u + 0.02 * rng.standard_normal(u.shape))
        v = np.asfortranarray(v + 0.02 * rng.standard_normal(v.shape))
    s.close()
    return out


@pytest.mark.parametrize("layout", ["curvilinear", "blockage"])
def test_small_scale_without_maps_bitwise(layout):
    """cu0 = 0: no map is iterated and the small scales stay zero; the
    filters, SmlSclBC, the small-scale Ppe and Project run all the same and
    every field equals the oracle's bit for bit."""
    for n_o, n_d, orc, dev in _run(layout, 0.0, 200.0, 0.004):
        assert n_d == n_o
        for k in orc:
            assert np.array_equal(dev[k], orc[k]), k


@pytest.mark.parametrize("layout,bnumc,dka", [("curvilinear", 200.0, 0.1), ("blockage", 50.0, 0.05)])
def test_small_scale_contracting_maps(layout, bnumc, dka):
    """Maps that contract (bnumc = 200, parse.f's value, on the curvilinear
    grid; bnumc = 50 on the blockage grid, whose weaker gradients leave the
    model idle at 200): the libm differences stay at rounding level, the
    small scales agree to 1e-11 of their largest value and the sweep counts
    are equal.  (On the oracle a 1e-15 relative change of u moves these
    outputs by under 1e-14 of their size.)"""
    res = _run(layout, 2.0, bnumc, dka)
    for n_o, n_d, orc, dev in res:
        assert n_d == n_o
        for k in orc:
            scale = max(float(np.max(np.abs(orc[k]))), 1e-300)
            assert float(np.max(np.abs(dev[k] - orc[k]))) <= 1e-11 * scale, k
    assert np.count_nonzero(res[-1][2]["uss"]) > 0


def test_small_scale_chaotic_maps():
    """bnumc = 5: the maps run near rmax, where one ulp grows to order one
    within the call's iterations.  The cells the model acts on (set by the
    large scales), the sweep counts of the small-scale Ppe, and the size of
    uss, vss, tss must still agree."""
    res = _run("curvilinear", 5.0, 5.0, 0.3, calls=2)
    for n_o, n_d, orc, dev in res:
        assert abs(n_d - n_o) <= 2
        for k in ("uss", "tss"):
            assert np.array_equal(dev[k] != 0.0, orc[k] != 0.0), k
            assert np.all(np.isfinite(dev[k]))
            ro = float(np.sqrt(np.mean(orc[k] ** 2)))
            rd = float(np.sqrt(np.mean(dev[k] ** 2)))
            assert ro > 0 and 0.5 * ro <= rd <= 2.0 * ro, (k, ro, rd)


@pytest.mark.parametrize("cu0,bnumc,tol", [(0.0, 200.0, 0.0), (2.0, 200.0, 1e-9)])
def test_small_scale_time_loop(cu0, bnumc, tol):
    """main.f's loop with nsmallscl = 1 driven through the drop-ins
    (wolfd2_gb300.atd.AtdLoop, the calling pattern of the Fortran driver)
    against the oracle's loop, from a developed lid-driven flow: bit for bit
    with the maps off (cu0 = 0), within 1e-9 of each field's size with
    contracting maps (bnumc = 200)."""
    from wolfd2_gb300.atd import AtdLoop
    case = deck.cavity(32, 800.0, 0.004, solver="rb_sor")
    dev = O.OracleRun(case)
    dev.step(40)
    fields = {k: dev.f[k].copy(order="F") for k in ("u", "v", "p", "t", "d")}
    case.atd = deck.SmallScaleParams(cu0=cu0, bnumc=bnumc, npsolver=deck.PPE_SOLVERS["rb_sor"], msorit=400,
                                     sorrel=1.3, fpu=300.0, fpv=300.0, fpt=200.0, pe=560.0)
    ref = O.OracleRun(case, fields=fields, cold_start=False)
    s = Solver.for_case(case, tuned=False)
    loop = AtdLoop(s, case, fields, ref._ap)
    assert loop.nsor_seed == ref.atd_nsor[0]
    ref.step(4)
    loop.step(4)
    assert [h[:2] for h in loop.history] == [h[:2] for h in ref.history]
    for k in ("u", "v", "p", "uss", "vss", "pss", "tss"):
        if tol == 0.0:
            assert np.array_equal(loop.f[k], ref.f[k]), k
        else:
            scale = max(float(np.max(np.abs(ref.f[k]))), 1e-300)
            assert float(np.max(np.abs(loop.f[k] - ref.f[k]))) <= tol * scale, k
    if cu0 > 0:
        assert np.abs(ref.f["uss"]).max() > 0
    s.close()
