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
