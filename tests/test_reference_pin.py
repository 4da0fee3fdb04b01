"""The oracle pinned to the reference's own source: a mechanical Fortran-77
-> C translation of src/momentum.f, src/pressure.f, src/utility.f,
src/bound_cond.f and src/grid.f (oracle/f77ref.py), sequenced as in
src/main.f (oracle/refrun.py), must give bit-identical fields and identical
iteration counts.  Skipped where neither the reference tree nor a previously
generated translation is present."""
import numpy as np
import pytest

import f77ref
import oracle as O
from wolfd2_gb300 import deck

if not (f77ref.available() or f77ref.build() is not None):
    pytest.skip("reference translation unavailable", allow_module_level=True)

import refrun  # noqa: E402

CASES = [
    ("cavity32_sor", lambda: deck.cavity(32, 100.0, 0.005, solver="sor")),
    ("cavity32_rb_sor", lambda: deck.cavity(32, 100.0, 0.005, solver="rb_sor")),
    ("cavity32_par_rb_sor", lambda: deck.cavity(32, 400.0, 0.004, solver="par_rb_sor")),
    ("rect_lsor", lambda: deck.cavity(40, 400.0, 0.004, solver="lsor", ny=24)),
    ("rect_rb_lsor", lambda: deck.cavity(36, 250.0, 0.004, solver="rb_lsor", ny=28)),
    ("channel_par_rb_lsor", lambda: deck.channel(48, 16, 500.0, 0.004, length=3.0, solver="par_rb_lsor")),
    ("channel_rb_sor", lambda: deck.channel(40, 20, 800.0, 0.003, length=2.0, solver="rb_sor")),
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_time_loop_bitwise(name, make):
    case = make()
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case)
    o = O.OracleRun(case)
    assert r.cold_nconv == o.cold_nconv
    for k in "uvp":
        assert np.array_equal(r.f[k], o.f[k]), f"cold start {k}"
    r.step(10)
    o.step(10)
    assert [h[:2] for h in r.history] == [h[:2] for h in o.history]
    for a, b in zip(r.history, o.history):
        assert a[2] == b[2]
    for k in "uvp":
        assert np.array_equal(r.f[k], o.f[k]), k


def test_blockage_and_porous_free_multiregion():
    """Three regions in i with an internal blockage and an outlet: exercises
    the blockage rows of Ppe/momentum and the region loops of the BCs."""
    text = ("number_of_regions 3 1\n i_borders 12 20\n j_borders\n"
            "blockage 2 1\n inlet 1 1 west nv 1.0\n outlet 3 1 east fd\n")
    case = deck.channel(32, 14, 300.0, 0.003, length=2.0, solver="rb_sor")
    case.regions = deck.parse_bc_section(text, case.nx, case.ny, re=case.params.re)
    case.bc_text = text
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case)
    o = O.OracleRun(case)
    r.step(6)
    o.step(6)
    assert [h[:2] for h in r.history] == [h[:2] for h in o.history]
    for k in "uvp":
        assert np.array_equal(r.f[k], o.f[k]), k


@pytest.mark.parametrize("layout", ["row", "quad", "curvi"])
def test_porous_regions_bitwise(layout):
    """PorosCoef and the porosity division of the convective coefficients
    (momentum.f:296-324, 621-649, 1115-1226): the oracle's time loop equals
    the translated reference's on porous layouts."""
    import porous_setup
    case = porous_setup.case(layout)
    assert (case.regions.nRegType == deck.RM_POROUS).sum() >= 2
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case)
    o = O.OracleRun(case)
    r.step(6)
    o.step(6)
    assert [h[:2] for h in r.history] == [h[:2] for h in o.history]
    for k in "uvp":
        assert np.array_equal(r.f[k], o.f[k]), k


def test_named_dt_diverges_at_1024():
    """At 1024x1024, Re=1000 the named dt=1e-3 drives the reference's own
    Newton-Kantorovich iteration to NaN in the first step (both in the
    translation and in the oracle); dt=2.5e-4 stays finite."""
    case = deck.cavity(1024, 1000.0, 1e-3, solver="rb_sor")
    u, v, p = deck.perturbation_ic(case, 1234)
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case, fields={"u": u, "v": v, "p": p}, cold_start=False)
    h = r.step(1)
    assert h[0] == -1 and not np.isfinite(r.f["u"]).all()


def _thermal_tables(th):
    return dict(ntrgtype=np.asfortranarray(th.nTRgType, np.int32),
                ntembdtp=np.asfortranarray(th.nTemBdTp, np.int32),
                dtrgval=np.asfortranarray(th.dTRgVal), dhgstval=np.asfortranarray(th.dHGSTval))


@pytest.mark.parametrize("pe", [50.0, 7.0])
def test_thermal_energy_bitwise(pe):
    """ThermEnergy (with its TempBoundCond and ConvCoef cases 3 and 6) on a
    curvilinear 3 x 2 region layout with fixed-temperature and heat-generating
    regions, fixed-temperature and heat-flux faces."""
    import thermal_setup
    case, th, f = thermal_setup.problem()
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case, cold_start=False)
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    for k in refrun.METRICS:
        assert np.array_equal(met[k], r.m[k]), k
    t_ref, t_or = f["t"].copy(order="F"), f["t"].copy(order="F")
    m = r.m
    r.R("thermenergy", nx=case.nx, ny=case.ny, nreg=r.tab["nreg"], nregbrd=r.tab["nregbrd"],
        **_thermal_tables(th), dk=0.004, pe=pe, dbcval=r.tab["dbcval"],
        rau=m["rau"], rbu=m["rbu"], rbv=m["rbv"], rgv=m["rgv"], djc=m["djc"],
        xeu=m["xeu"], yeu=m["yeu"], xzv=m["xzv"], yzv=m["yzv"],
        xec=m["xec"], yec=m["yec"], xzc=m["xzc"], yzc=m["yzc"],
        un=f["un"], vn=f["vn"], u=f["u"], v=f["v"], tn=f["tn"], t=t_ref)
    o.therm_energy(case.nx, case.ny, case.regions, th, 0.004, pe, met, f["un"], f["vn"], f["u"], f["v"],
                   f["tn"], t_or)
    assert np.isfinite(t_or).all()
    assert np.array_equal(t_ref, t_or)


def test_temp_bound_cond_and_eq_state_bitwise():
    import thermal_setup
    case, th, f = thermal_setup.problem(seed=9)
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case, cold_start=False)
    o = O.Oracle(case.nx + 1, case.ny + 1)
    a, b = f["t"].copy(order="F"), f["t"].copy(order="F")
    r.R("tempboundcond", nx=case.nx, ny=case.ny, nreg=r.tab["nreg"], nregbrd=r.tab["nregbrd"],
        **{k: v for k, v in _thermal_tables(th).items() if k != "dhgstval"}, dbcval=r.tab["dbcval"], t=a)
    o.temp_bound_cond(case.nx, case.ny, case.regions, th, b)
    assert np.array_equal(a, b)
    da, db = r.z(), r.z()
    # temperatures in [0, 1] of the reference scale, pressure of either sign
    t = np.asfortranarray(0.5 + 0.4 * np.tanh(f["tn"]))
    kw = dict(uref=1.3, densref=1.1, tmax=350.0, tref=290.0, rconst=287.0)
    r.R("eqstate", nx=case.nx, ny=case.ny, **kw, p=f["p"], t=t, den=da)
    o.eq_state(case.nx, case.ny, kw["uref"], kw["densref"], kw["tmax"], kw["tref"], kw["rconst"],
               f["p"], t, db)
    assert np.array_equal(da, db) and np.count_nonzero(da) > 0


@pytest.mark.parametrize("nmeiter,eqstate", [(1, False), (3, True), (6, True)])
def test_heated_cavity_time_loop_bitwise(nmeiter, eqstate):
    """The time loop with the energy equation: momentum/energy iterations
    (main.f:736-879) with ThermEnergy, EqState feeding the buoyancy term of
    YMomentum, and TempBoundCond after them."""
    case = deck.heated_cavity(24, 500.0, 0.004, nmeiter=nmeiter, dmeittol=1e-7, eqstate=eqstate)
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case)
    o = O.OracleRun(case)
    r.step(8)
    o.step(8)
    assert [h[:2] for h in r.history] == [h[:2] for h in o.history]
    for a, b in zip(r.history, o.history):
        assert a[2] == b[2]
    for k in ("u", "v", "p", "t", "d"):
        assert np.array_equal(r.f[k], o.f[k]), k
    assert np.abs(o.f["t"]).max() > 0.1
    if eqstate:
        assert np.abs(o.f["d"]).max() > 1e-3


def test_multiregion_thermal_time_loop_bitwise():
    """The time loop with the energy equation on the curvilinear 3 x 2
    layout (fixed-temperature and heat-generating regions)."""
    import thermal_setup
    case = thermal_setup.loop_case()
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case)
    o = O.OracleRun(case)
    r.step(5)
    o.step(5)
    assert [h[:2] for h in r.history] == [h[:2] for h in o.history]
    for a, b in zip(r.history, o.history):
        assert a[2] == b[2]
    for k in ("u", "v", "p", "t", "d"):
        assert np.array_equal(r.f[k], o.f[k]), k


@pytest.mark.parametrize("layout", ["heated", "multiregion"])
def test_thermal_loop_with_filter_bitwise(layout):
    """Filter of t after the momentum/energy iterations (main.f:889-893;
    utility.f's scalar branch skips the regions whose nTRgType equals 1)."""
    import thermal_setup
    if layout == "heated":
        case = deck.heated_cavity(24, 500.0, 0.004, nmeiter=2, dmeittol=1e-7)
    else:
        case = thermal_setup.loop_case(nmeiter=2)
    case.tparams.nfiltt = 1
    case.tparams.fpt = 20.0
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case)
    o = O.OracleRun(case)
    r.step(5)
    o.step(5)
    assert [h[:2] for h in r.history] == [h[:2] for h in o.history]
    for a, b in zip(r.history, o.history):
        assert a[2] == b[2]
    for k in ("u", "v", "p", "t", "d"):
        assert np.array_equal(r.f[k], o.f[k]), k


@pytest.mark.parametrize("solver", ["rb_sor", "rb_lsor"])
def test_curvilinear_multiregion_time_loop_bitwise(solver):
    """The plain time loop on the curvilinear 3 x 2 layout with lcartes = 0:
    RhsPpe forms the cross terms before every sweep (pressure.f:362-375)."""
    import thermal_setup
    case = thermal_setup.curvilinear_case()
    case.params.npsolver = deck.PPE_SOLVERS[solver]
    case.params.msorit = 300
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case)
    o = O.OracleRun(case)
    r.step(5)
    o.step(5)
    assert [h[:2] for h in r.history] == [h[:2] for h in o.history]
    for k in "uvp":
        assert np.array_equal(r.f[k], o.f[k]), k


def _atd_layout(name):
    """(case, thermal tables, large-scale u, v, t) for the small-scale pin."""
    import thermal_setup
    if name == "blockage":
        case = thermal_setup.blockage_case()
        th = deck.Thermal.empty()
        rng = np.random.default_rng(3)
        o = O.Oracle(case.nx + 1, case.ny + 1)
        u, v, p = deck.perturbation_ic(case, 5, amp=0.3)
        t = np.asfortranarray(rng.uniform(0.0, 1.0, size=u.shape))
        return case, th, u, v, t
    case, th, f = thermal_setup.problem()
    case.params.lcartes = 0
    t = np.asfortranarray(0.5 + 0.4 * np.tanh(f["tn"]))
    return case, th, np.asfortranarray(f["u"]), np.asfortranarray(f["v"]), t


@pytest.mark.parametrize("layout,solver,cu0,dka,bnumc", [
    ("curvilinear", "rb_sor", 5.0, 0.3, 5.0),
    ("curvilinear", "sor", 0.8, 0.05, 8.0),
    ("curvilinear", "rb_sor", 2.0, 0.1, 200.0),   # parse.f's bnumc: rmap ~ 1e-6
    ("curvilinear", "rb_lsor", 0.0, 0.004, 200.0),   # parse.f's cu0 = 0: no maps
    ("blockage", "rb_sor", 3.0, 0.2, 5.0),
])
def test_small_scale_bitwise(layout, solver, cu0, dka, bnumc):
    """SmallScale (small_scale.f:31-578) with SmlSclBC, its Filters, Ppe and
    Project: the initial call and three more, against the translated source;
    the map iterates and cell areas carry over between calls in both.  A
    small bnumc drives the maps into their chaotic range (rmap near rmax)."""
    case, th, u, v, t = _atd_layout(layout)
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case, cold_start=False)
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    re, pe, npsolver = 1000.0, 700.0, deck.PPE_SOLVERS[solver]
    ap = O.AtdParams.make(dka=dka, re=re, pe=pe, npsolver=npsolver, msorit=300,
                          lcartes=case.params.lcartes, cu0=cu0, sortol=1e-9, sorrel=1.2,
                          fp=(400.0, 300.0, 0.0, 200.0), bnumc=bnumc)
    atd = O.SmallScale(o, case.nx, case.ny, case.regions, th, met, ap)
    tb, m = r.tab, r.m
    ref = {k: o.field() for k in ("uss", "vss", "pss", "tss")}
    orc = {k: o.field() for k in ("uss", "vss", "pss", "tss")}
    rng = np.random.default_rng(11)
    for call in range(4):
        r.R("smallscale", nx=case.nx, ny=case.ny, initflg=0 if call == 0 else 1, nthermen=1,
            lcartesgrid=case.params.lcartes, nreg=tb["nreg"], nregbrd=tb["nregbrd"],
            nregtype=tb["nregtype"], nmombdtp=tb["nmombdtp"], **{k: w for k, w in
                                                                 _thermal_tables(th).items()
                                                                 if k != "dhgstval"},
            nppesolver=npsolver, msorit=300, dlref=1.0, uref=1.0, tref=300.0, tmax=330.0,
            dka=dka, re=re, pe=pe, sortol=1e-9, sorrel=1.2,
            fp=np.array([400.0, 300.0, 0.0, 200.0]), cu0=cu0, tscoef=1.0, hscoef=1.0,
            temcoef=1.0, bnumc=bnumc, rmax=0.95, rlc=5.0, dbcval=tb["dbcval"],
            **{k: m[k] for k in ("rau", "rbu", "rbv", "rgv", "dju", "djv", "djc", "xeu", "yeu",
                                 "xzv", "yzv", "xzu", "yzu", "xev", "yev", "xec", "yec", "xzc",
                                 "yzc")},
            u1=u, v1=v, t1=t, **ref)
        atd(0 if call == 0 else 1, u, v, t, orc["uss"], orc["vss"], orc["pss"], orc["tss"])
        for k in ref:
            assert np.array_equal(ref[k], orc[k], equal_nan=True), (call, k)
        # the next call sees slightly different large scales
        u = np.asfortranarray(u + 0.02 * rng.standard_normal(u.shape))
        v = np.asfortranarray(v + 0.02 * rng.standard_normal(v.shape))
    if cu0 > 0 and bnumc < 10:
        assert np.count_nonzero(orc["uss"]) > 0 and np.count_nonzero(orc["tss"]) > 0
        assert np.abs(orc["tss"]).max() > 1e-6
    elif cu0 == 0:
        assert not orc["uss"].any() and not orc["tss"].any()


@pytest.mark.parametrize("outlet", ["fd", "mc"])
def test_sml_scl_bc_bitwise(outlet):
    """SmlSclBC (bound_cond.f:1211-1500) on a channel with either outlet
    type (BM_OUTLT1, BM_OUTLT2) and the heated cavity's temperature faces,
    and on the thermal 3 x 2 layout (a fixed-temperature region)."""
    import thermal_setup
    rng = np.random.default_rng(7)
    hc = deck.heated_cavity(8, 100.0, 0.01)
    for case, th in ((deck.channel(30, 12, 200.0, 0.003, outlet=outlet), hc.thermal),
                     thermal_setup.problem()[:2]):
        f77ref.build(case.nx + 1, case.ny + 1)
        r = refrun.RefRun(case, cold_start=False)
        o = O.Oracle(case.nx + 1, case.ny + 1)
        if case.regions.nReg[0] * case.regions.nReg[1] == 1:
            th = deck.Thermal.empty()
            th.nTemBdTp[0, 0, :] = hc.thermal.nTemBdTp[0, 0, :]
        a = {k: np.asfortranarray(rng.standard_normal((case.nx + 2, case.ny + 2))) for k in "uvpt"}
        b = {k: w.copy(order="F") for k, w in a.items()}
        tb = r.tab
        tt = _thermal_tables(th)
        r.R("smlsclbc", nx=case.nx, ny=case.ny, nreg=tb["nreg"], nregbrd=tb["nregbrd"],
            nregtype=tb["nregtype"], nmombdtp=tb["nmombdtp"], ntrgtype=tt["ntrgtype"],
            ntembdtp=tt["ntembdtp"], dbcval=tb["dbcval"], u=a["u"], v=a["v"], p=a["p"], t=a["t"])
        o.sml_scl_bc(case.nx, case.ny, case.regions, th, b["u"], b["v"], b["p"], b["t"])
        for k in "uvpt":
            assert np.array_equal(a[k], b[k]), k


def _atd_case(name):
    import thermal_setup
    if name == "heated":
        case = deck.heated_cavity(24, 500.0, 0.004, nmeiter=2, dmeittol=1e-7, lid=1.0)
        pe = case.tparams.pe
    elif name == "multiregion":
        case = thermal_setup.loop_case(nmeiter=2)
        case.params.re, case.tparams.pe = 1500.0, 1050.0
        pe = case.tparams.pe
    else:   # no energy equation: SmallScale still takes the (empty) thermal tables
        case = deck.cavity(32, 800.0, 0.004, solver="rb_sor")
        pe = 560.0
    case.atd = deck.SmallScaleParams(cu0=0.5, bnumc=5.0, npsolver=deck.PPE_SOLVERS["rb_sor"],
                                     msorit=400, sorrel=1.3, fpu=300.0, fpv=300.0, fpt=200.0,
                                     pe=pe)
    return case


@pytest.mark.parametrize("name", ["plain", "heated", "multiregion"])
def test_time_loop_with_small_scales_bitwise(name):
    """The time loop with nsmallscl = 1 (main.f:645-664, 708-730, 898-940):
    the small scales added to level n, removed from level n+1, recomputed by
    SmallScale (chaotic maps live) and added back, against the translation."""
    case = _atd_case(name)
    f77ref.build(case.nx + 1, case.ny + 1)
    # a developed lid-driven field (40 steps of the pinned loop without the
    # model): from rest the sub-grid Peclet number stays below its
    # threshold (3) everywhere and the model adds nothing
    atd, case.atd = case.atd, None
    dev = O.OracleRun(case)
    dev.step(40)
    case.atd = atd
    fields = {k: dev.f[k].copy(order="F") for k in ("u", "v", "p", "t", "d")}
    r = refrun.RefRun(case, fields=fields)
    o = O.OracleRun(case, fields=fields)
    for k in ("uss", "vss", "pss", "tss"):
        assert np.array_equal(r.f[k], o.f[k]), ("init", k)
    r.step(5)
    o.step(5)
    assert [h[:2] for h in r.history] == [h[:2] for h in o.history]
    for a, b in zip(r.history, o.history):
        assert a[2] == b[2]
    for k in ("u", "v", "p", "t", "uss", "vss", "pss", "tss"):
        assert np.array_equal(r.f[k], o.f[k]), k
    assert np.abs(o.f["uss"]).max() > 1e-6 and np.abs(o.f["tss"]).max() > 1e-6
