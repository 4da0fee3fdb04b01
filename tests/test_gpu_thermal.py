"""GPU parity of the thermal drop-ins (ThermEnergy, TempBoundCond, EqState)
and of the buoyancy term of nAuxMomentum against the CPU oracle: bit-for-bit
equal fields on a curvilinear 3 x 2 region layout with fixed-temperature and
heat-generating regions and fixed-temperature / heat-flux faces."""
import numpy as np
import pytest

import oracle as O
import thermal_setup
from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import Solver, W2Error

pytestmark = pytest.mark.gpu


def _setup(seed=5):
    case, th, f = thermal_setup.problem(seed=seed)
    s = Solver.for_case(case, tuned=False)
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    return case, th, f, s, o, met


@pytest.mark.parametrize("pe,dk", [(50.0, 0.004), (3.0, 0.02)])
def test_therm_energy_bitwise(pe, dk):
    case, th, f, s, o, met = _setup()
    tg, to = f["t"].copy(order="F"), f["t"].copy(order="F")
    s.ThermEnergy(th, dk, pe, f["un"], f["vn"], f["u"], f["v"], f["tn"], tg)
    o.therm_energy(case.nx, case.ny, case.regions, th, dk, pe, met, f["un"], f["vn"], f["u"], f["v"],
                   f["tn"], to)
    assert np.isfinite(to).all()
    assert np.array_equal(tg, to), float(np.max(np.abs(tg - to)))
    s.close()


def test_therm_energy_single_region_cavity():
    """One region (the whole cavity), hot west wall, adiabatic others, a heat
    source everywhere: the chain couples every row through its end rows."""
    case = deck.cavity(48, 100.0, 0.005, solver="rb_sor")
    th = deck.Thermal.empty()
    th.nTRgType[0, 0] = deck.RT_HEATGN
    th.dHGSTval[0, 0] = 0.05
    th.nTemBdTp[0, 0, :] = (deck.BT_TEMPER, deck.BT_HTFLUX, deck.BT_HTFLUX, deck.BT_HTFLUX)
    case.regions.dBCVal[0, 0, deck.WEST - 1, deck.VAR_T - 1] = 1.0
    s = Solver.for_case(case, tuned=False)
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    u, v, p = deck.perturbation_ic(case, 3, amp=0.05)
    rng = np.random.default_rng(4)
    tn = np.asfortranarray(rng.uniform(0.0, 1.0, size=u.shape))
    tg, to = tn.copy(order="F"), tn.copy(order="F")
    s.ThermEnergy(th, 0.005, 70.0, u, v, u, v, tn, tg)
    o.therm_energy(case.nx, case.ny, case.regions, th, 0.005, 70.0, met, u, v, u, v, tn, to)
    assert np.array_equal(tg, to)
    s.close()


def test_temp_bound_cond_and_eq_state_bitwise():
    case, th, f, s, o, met = _setup(seed=9)
    a, b = f["t"].copy(order="F"), f["t"].copy(order="F")
    s.TempBoundCond(th, a)
    o.temp_bound_cond(case.nx, case.ny, case.regions, th, b)
    assert np.array_equal(a, b)
    t = np.asfortranarray(0.5 + 0.4 * np.tanh(f["tn"]))
    kw = (1.3, 1.1, 350.0, 290.0, 287.0)
    dg, do = np.asfortranarray(f["u"].copy()), np.asfortranarray(f["u"].copy())
    s.EqState(*kw, f["p"], t, dg)
    o.eq_state(case.nx, case.ny, *kw, f["p"], t, do)
    assert np.array_equal(dg, do) and np.count_nonzero(do[2:case.nx + 1, 2:case.ny + 1]) > 0
    s.close()


def test_bad_thermal_flag_is_an_error():
    case, th, f, s, o, met = _setup()
    th.nTemBdTp[0, 0, 0] = 7
    with pytest.raises(W2Error):
        s.TempBoundCond(th, f["t"].copy(order="F"))
    s.close()


def _momentum_inputs(o, case, f, amp=0.1):
    """Smooth velocities made consistent with the boundary conditions, and
    the densities of EqState at two temperatures."""
    nx, ny = case.nx, case.ny
    u, v = np.asfortranarray(amp * f["u"]), np.asfortranarray(amp * f["v"])
    o.vel_bound_cond(nx, ny, case.regions, u, v)
    t = np.asfortranarray(0.5 + 0.4 * np.tanh(f["tn"]))
    tn = np.asfortranarray(0.5 + 0.4 * np.tanh(f["t"]))
    den, denn = o.field(), o.field()
    o.eq_state(nx, ny, 1.0, 1.0, 320.0, 290.0, 287.0, f["p"], t, den)
    o.eq_state(nx, ny, 1.0, 1.0, 320.0, 290.0, 287.0, f["p"], tn, denn)
    return u, v, den, denn


@pytest.mark.parametrize("buoyant", [False, True])
def test_momentum_multiregion_curvilinear(buoyant):
    """nAuxMomentum on the 3 x 2 curvilinear layout, with and without the
    buoyancy term of the density from EqState."""
    case, th, f, s, o, met = _setup()
    nx, ny = case.nx, case.ny
    u, v, den, denn = _momentum_inputs(o, case, f)
    assert np.count_nonzero(den) > 0
    prm = dataclasses_replace(case.params, fr=0.37)
    dg, dng = (den, denn) if buoyant else (None, None)
    do, dno = (den, denn) if buoyant else (o.field(), o.field())
    usg, vsg = u.copy(order="F"), v.copy(order="F")
    uso, vso = u.copy(order="F"), v.copy(order="F")
    ng = s.nAuxMomentum(prm.mqiter, prm.dk, prm.re, prm.fr, prm.qtol, dg, dng, u, v, usg, vsg)
    no = o.naux_momentum(nx, ny, case.regions, prm, met, do, dno, u, v, uso, vso)
    assert ng == no and ng > 0
    assert np.array_equal(usg, uso) and np.array_equal(vsg, vso)
    if buoyant:
        # the term is live: zero density gives a different v
        us0, vs0 = u.copy(order="F"), v.copy(order="F")
        s.nAuxMomentum(prm.mqiter, prm.dk, prm.re, prm.fr, prm.qtol, None, None, u, v, us0, vs0)
        assert not np.array_equal(vs0, vsg)
    s.close()


def test_momentum_divergence_reported_like_reference():
    """Velocities far from their boundary values drive the Newton-Kantorovich
    iteration to NaN: the run is not converged (-1), as in the reference,
    and the NaN fields agree with the oracle's."""
    case, th, f, s, o, met = _setup()
    nx, ny = case.nx, case.ny
    u, v, p = deck.perturbation_ic(case, 11, amp=0.05)
    prm = case.params
    usg, vsg = u.copy(order="F"), v.copy(order="F")
    uso, vso = u.copy(order="F"), v.copy(order="F")
    ng = s.nAuxMomentum(prm.mqiter, prm.dk, prm.re, prm.fr, prm.qtol, None, None, u, v, usg, vsg)
    no = o.naux_momentum(nx, ny, case.regions, prm, met, o.field(), o.field(), u, v, uso, vso)
    assert no == -1 and ng == -1
    assert np.array_equal(usg, uso, equal_nan=True) and np.array_equal(vsg, vso, equal_nan=True)
    s.close()


def dataclasses_replace(p, **kw):
    import dataclasses
    return dataclasses.replace(p, **kw)


def _filtered(case):
    case.tparams.nfiltt = 1
    case.tparams.fpt = 20.0
    return case


def _loop_cases():
    return {
        "heated1": lambda: deck.heated_cavity(32, 500.0, 0.004, nmeiter=1, eqstate=False),
        "heated3": lambda: deck.heated_cavity(32, 500.0, 0.004, nmeiter=3, dmeittol=1e-7),
        "heated6_lid": lambda: deck.heated_cavity(40, 300.0, 0.004, nmeiter=6, dmeittol=1e-6, lid=1.0),
        "multiregion": lambda: thermal_setup.loop_case(),
        "multiregion_filter_t": lambda: _filtered(thermal_setup.loop_case(nmeiter=2)),
    }


def test_filter_t_bitwise():
    """Filter of the temperature on the 3 x 2 layout: the heat-generating
    region (nTRgType 1) is skipped, as the reference's test skips it."""
    case, th, f, s, o, met = _setup()
    tg, to = f["t"].copy(order="F"), f["t"].copy(order="F")
    s.FilterT(th, 20.0, tg)
    o.filter_t(case.nx, case.ny, case.regions, th, 20.0, to)
    assert np.array_equal(tg, to) and not np.array_equal(tg, f["t"])
    s.close()


@pytest.mark.parametrize("name", sorted(_loop_cases()))
@pytest.mark.parametrize("graph", [False, True])
def test_thermal_time_loop_matches_oracle(name, graph):
    """The device-resident step with the energy equation (momentum/energy
    iterations ending on the device, ThermEnergy, EqState, buoyancy,
    TempBoundCond) against the oracle's time loop: bit-identical fields,
    temperatures, densities and iteration counts."""
    case = _loop_cases()[name]()
    o = O.OracleRun(case)
    s = Solver.for_case(case, tuned=False)
    s.graph(graph)
    s.load_fields(o.f["u"], o.f["v"], o.f["p"])
    s.load_thermal(o.f["t"], o.f["d"])
    nsteps = 6
    hist = s.step(case.params, 3) + s.step(case.params, 3)
    o.step(nsteps)
    assert [(h[0], h[1]) for h in hist] == [h[:2] for h in o.history]
    for h, oh in zip(hist, o.history):
        assert tuple(h[2]) == tuple(oh[2])
    u, v, p = s.store_fields()
    t, dd = s.store_thermal()
    for name_, g, r in zip("uvptd", (u, v, p, t, dd), (o.f["u"], o.f["v"], o.f["p"], o.f["t"], o.f["d"])):
        assert np.array_equal(g, r), (name_, float(np.max(np.abs(g - r))))
    assert np.abs(t).max() > 0.1
    s.close()


def test_deck_driven_thermal_run(tmp_path):
    """A reference-style deck (thermal energy, buoyancy, Filter of t, a fluid
    table) read by read_deck and stepped on the device equals the oracle's
    time loop on the same case."""
    c = deck.cavity(32, 100.0, 0.01)
    deck.write_grid_plot3d(str(tmp_path / "grid.xyz"), c.x, c.y)
    (tmp_path / "fluid.dat").write_text(
        "fluid air01 gasconstant 287.0\n280 1.2 1000 0.010 0.025 0.70\n320 1.0 1000 0.012 0.027 0.72\nend\n")
    (tmp_path / "input.dat").write_text(
        "section input_parameters\n grid_file grid.xyz cartesian_grid\n thermal_energy\n buoyancy\n"
        " time_step_size 0.004\n ref_temperature 300\n max_ref_temperature 330\n"
        " fluid_prop_file fluid.dat\n max_me_iter 2\n me_tolerance 1d-9\n filter_t 50.0\n"
        " ppe_solver rb_sor\n max_sor_iter 400\nend section\n\n"
        "section boundary_conditions\n number_of_regions 1 1\n i_borders\n j_borders\n"
        " wall 1 1 north tv 1.0\n wall 1 1 west t 330\n wall 1 1 east t 300\nend section\n")
    case = deck.read_deck(str(tmp_path / "input.dat"))
    o = O.OracleRun(case)
    o.step(4)
    s = Solver.for_case(case, tuned=False)
    z = s.field()
    s.load_fields(z, z, z)
    s.cold_start(case.params)
    hist = s.step(case.params, 4)
    assert [(h[0], h[1]) for h in hist] == [h[:2] for h in o.history]
    u, v, p = s.store_fields()
    t, d = s.store_thermal()
    for nm, g in zip("uvptd", (u, v, p, t, d)):
        assert np.array_equal(g, o.f[nm]), nm
    assert np.abs(t).max() > 0.1
    s.close()
