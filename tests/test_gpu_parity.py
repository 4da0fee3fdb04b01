"""GPU parity: every drop-in entry point and the device-resident time loop
against the CPU oracle on the same inputs.  The library evaluates the
reference expressions operation by operation (no FMA contraction) and solves
the concatenated chains with the exact sequential recurrence, so the bar is
bit-for-bit equality of fields and equal iteration counts; the relative
tolerance 1e-10 of the plain FP64 path is asserted as well."""
import numpy as np
import pytest

import oracle as O
from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import Solver

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def smooth_field(rng, nx, ny, amp=1.0, modes=4):
    f = np.zeros((nx + 2, ny + 2), order="F")
    x = np.linspace(0, 1, nx + 2)[:, None]
    y = np.linspace(0, 1, ny + 2)[None, :]
    for _ in range(modes):
        k, l = rng.integers(1, 6, size=2)
        f += amp * rng.normal() * np.sin(k * np.pi * x + rng.uniform(0, 6)) * np.cos(l * np.pi * y)
    return f


def fields_for(case, seed, amp=0.3):
    rng = np.random.default_rng(seed)
    out = {}
    for name in ("u", "v", "p"):
        a = np.zeros((case.nx + 2, case.ny + 2), order="F")
        a[...] = smooth_field(rng, case.nx, case.ny, amp)
        out[name] = a
    return out


def oracle_setup(case):
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    return o, met


CASES = {
    "cavity33": lambda: deck.cavity(32, 100.0, 0.005, solver="rb_sor"),
    "cavity_rect": lambda: deck.cavity(40, 400.0, 0.004, solver="rb_sor", ny=24),
    "channel": lambda: deck.channel(48, 16, 500.0, 0.004, length=3.0, solver="rb_sor"),
    "channel_mc": lambda: deck.channel(40, 20, 800.0, 0.004, length=2.5, solver="rb_sor", outlet="mc"),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    return CASES[request.param]()


def test_grid_metric_matches_oracle(case):
    s = Solver(case.nx, case.ny, case.regions)
    met = s.grid_metric(case.x, case.y, want=True)
    _, omet = oracle_setup(case)
    for name, arr in met.items():
        assert np.array_equal(arr, omet[name]), name


def test_boundary_conditions(case):
    o, met = oracle_setup(case)
    s = Solver.for_case(case)
    f = fields_for(case, 1)
    u, v, p = (f[k].copy(order="F") for k in "uvp")
    gu, gv, gp = u.copy(order="F"), v.copy(order="F"), p.copy(order="F")
    o.vel_bound_cond(case.nx, case.ny, case.regions, u, v)
    s.VelBoundCond(gu, gv)
    assert np.array_equal(gu, u) and np.array_equal(gv, v)
    o.pres_bound_cond(case.nx, case.ny, case.regions, p)
    s.PresBoundCond(gp)
    assert np.array_equal(gp, p)
    o.vel_outflow_bcs(case.nx, case.ny, case.regions, u, v)
    s.VelOutflowBCs(gu, gv)
    assert np.array_equal(gu, u) and np.array_equal(gv, v)


def test_project_and_norm(case):
    o, met = oracle_setup(case)
    s = Solver.for_case(case)
    f = fields_for(case, 2)
    u, v, p = (f[k].copy(order="F") for k in "uvp")
    gu, gv = u.copy(order="F"), v.copy(order="F")
    o.project(case.nx, case.ny, case.regions, case.params.dk, met, p, u, v)
    s.Project(case.params.dk, p, gu, gv)
    assert np.array_equal(gu, u) and np.array_equal(gv, v)
    assert s.DiffMaxNorm(f["u"], u) == o.diff_max_norm(case.nx, case.ny, f["u"], u)


@pytest.mark.parametrize("solver", [1, 2, 3, 4, 5, 6])
def test_ppe_solvers(case, solver):
    if solver in (1, 2) and case.nx * case.ny > 3000:
        pytest.skip("sequential solvers checked on the small cases")
    o, met = oracle_setup(case)
    s = Solver.for_case(case)
    f = fields_for(case, 3, amp=0.05)
    u, v = f["u"], f["v"]
    p = f["p"].copy(order="F")
    o.vel_bound_cond(case.nx, case.ny, case.regions, u, v)
    o.pres_bound_cond(case.nx, case.ny, case.regions, p)
    gp = p.copy(order="F")
    prm = case.params
    n_o = o.ppe(case.nx, case.ny, case.regions, prm, met, u, v, p, npsolver=solver, msorit=300)
    n_g = s.Ppe(True, solver, 300, prm.dk, prm.sortol, prm.sorrel, u, v, gp)
    assert n_g == n_o
    assert np.array_equal(gp, p), rel_err(gp, p)


def test_ppe_non_cartesian(case):
    o, met = oracle_setup(case)
    s = Solver.for_case(case)
    f = fields_for(case, 4, amp=0.05)
    p = f["p"].copy(order="F")
    gp = p.copy(order="F")
    prm = case.params
    n_o = o.ppe(case.nx, case.ny, case.regions, deck.RunParams(**{**prm.__dict__, "lcartes": 0}),
                met, f["u"], f["v"], p, npsolver=5, msorit=100)
    n_g = s.Ppe(False, 5, 100, prm.dk, prm.sortol, prm.sorrel, f["u"], f["v"], gp)
    assert n_g == n_o and np.array_equal(gp, p)


def test_naux_momentum(case):
    o, met = oracle_setup(case)
    s = Solver.for_case(case)
    f = fields_for(case, 5, amp=0.2)
    un, vn = f["u"], f["v"]
    o.vel_bound_cond(case.nx, case.ny, case.regions, un, vn)
    us, vs = un.copy(order="F"), vn.copy(order="F")
    gus, gvs = us.copy(order="F"), vs.copy(order="F")
    z = o.field()
    prm = case.params
    n_o = o.naux_momentum(case.nx, case.ny, case.regions, prm, met, z, z, un, vn, us, vs)
    n_g = s.nAuxMomentum(prm.mqiter, prm.dk, prm.re, prm.fr, prm.qtol, None, None, un, vn, gus, gvs)
    assert n_g == n_o
    assert np.array_equal(gus, us), rel_err(gus, us)
    assert np.array_equal(gvs, vs), rel_err(gvs, vs)


def test_time_loop_matches_oracle(case):
    ref = O.OracleRun(case)
    ref.step(12)
    s = Solver.for_case(case)
    z = s.field()
    s.load_fields(z, z, z)
    assert s.cold_start(case.params) == ref.cold_nconv
    hist = s.step(case.params, 12)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in ref.history]
    for a, b in zip(hist, ref.history):
        assert a[2][:3] == b[2][:3]
    u, v, p = s.store_fields()
    for name, g in (("u", u), ("v", v), ("p", p)):
        assert rel_err(g, ref.f[name]) <= REL_TOL
        assert np.array_equal(g, ref.f[name]), name


def test_cavity64_lexicographic_sor_60_steps():
    """The 64x64 cavity (Re=100, dt=0.005, point SOR) against the oracle
    field by field for its first 60 steps.  All 500 steps of this
    configuration run in tests/test_gpu_golden.py against the fixture made
    from the translated reference source (per-field SHA-256)."""
    case = deck.cavity(64, 100.0, 0.005, solver="sor")
    ref = O.OracleRun(case)
    ref.step(60)
    s = Solver.for_case(case)
    z = s.field()
    s.load_fields(z, z, z)
    s.cold_start(case.params)
    hist = s.step(case.params, 60)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in ref.history]
    u, v, p = s.store_fields()
    for name, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, ref.f[name]), (name, rel_err(g, ref.f[name]))


@pytest.mark.parametrize("ncomp", [1, 2])
def test_velocity_filter_bitwise(case, ncomp):
    """Filter of u (ncomp 1) or v (ncomp 2), utility.f:33-247: the Shuman
    filter (sum of the four neighbours + fp*q)/(fp + 4) on the points each
    region's loops cover, every other point unchanged."""
    o, _ = oracle_setup(case)
    s = Solver.for_case(case)
    f = fields_for(case, 31 + ncomp)
    q = f["u" if ncomp == 1 else "v"]
    gq, oq = q.copy(order="F"), q.copy(order="F")
    s.Filter(ncomp, 20.0, gq)
    o.filter(case.nx, case.ny, ncomp, case.regions, 20.0, oq)
    assert np.array_equal(gq, oq) and not np.array_equal(gq, q)


def test_time_loop_with_velocity_filter(case):
    """main.f:783-791: filter_u and filter_v on, the starred velocities
    filtered inside every step before the boundary conditions and Ppe;
    the device loop bit-identical to the oracle's."""
    import dataclasses
    case = dataclasses.replace(case, params=dataclasses.replace(case.params, nfiltu=1, nfiltv=1,
                                                                 fpu=40.0, fpv=60.0))
    ref = O.OracleRun(case)
    ref.step(6)
    s = Solver.for_case(case)
    z = s.field()
    s.load_fields(z, z, z)
    assert s.cold_start(case.params) == ref.cold_nconv
    hist = s.step(case.params, 6)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in ref.history]
    u, v, p = s.store_fields()
    for name, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, ref.f[name]), (name, rel_err(g, ref.f[name]))


@pytest.mark.parametrize("wide", [False, True])
@pytest.mark.parametrize("sorrel", [1.0, 1.9])
@pytest.mark.parametrize("sortol", [1e-8, 3e-6, 1e-5, 2e-5])
@pytest.mark.parametrize("msorit", [301, 300])
def test_tiled_red_black_sweeps(sortol, msorit, sorrel, wide):
    """Two sweeps per barrier on shared-memory tiles (forced on a small
    grid): bit-identical p and nSorConv for stopping points on either sweep
    of a pair, for odd and even msorit, with and without over-relaxation, in
    512- and 1024-thread blocks."""
    case = deck.cavity(128, 400.0, 0.002, solver="rb_sor", ny=64)
    o, met = oracle_setup(case)
    s = Solver.for_case(case)
    s.tune(blocks_per_sm=-2)
    if wide:
        s.tune(blocks_per_sm=-3)   # 1024-thread blocks
    f = fields_for(case, 9, amp=0.05)
    u, v = f["u"], f["v"]
    p = f["p"].copy(order="F")
    o.vel_bound_cond(case.nx, case.ny, case.regions, u, v)
    o.pres_bound_cond(case.nx, case.ny, case.regions, p)
    gp = p.copy(order="F")
    prm = deck.RunParams(**{**case.params.__dict__, "sortol": sortol, "sorrel": sorrel})
    n_o = o.ppe(case.nx, case.ny, case.regions, prm, met, u, v, p, npsolver=5, msorit=msorit)
    n_g = s.Ppe(True, 5, msorit, prm.dk, sortol, sorrel, u, v, gp)
    assert n_g == n_o
    assert np.array_equal(gp, p), rel_err(gp, p)


def test_tiled_time_loop_512():
    """The benchmark's code path (tiled sweeps, unit stencil) over a few
    steps of a 512x512 cavity from the seeded perturbation."""
    case = deck.cavity(512, 1000.0, 2.5e-4, solver="rb_sor")
    u0, v0, p0 = deck.perturbation_ic(case, 1234)
    ref = O.OracleRun(case, fields={"u": u0, "v": v0, "p": p0}, cold_start=False)
    ref.step(2)
    s = Solver.for_case(case)
    s.load_fields(u0, v0, p0)
    hist = s.step(case.params, 2)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in ref.history]
    u, v, p = s.store_fields()
    for name, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, ref.f[name]), (name, rel_err(g, ref.f[name]))


@pytest.mark.parametrize("seg,warm", [(8, 1), (13, 4), (27, 64), (97, 2), (4096, 64)])
def test_chain_segments_exact(seg, warm):
    """nAuxMomentum bit-identical for segment lengths that do and do not
    divide the chains and for warm-ups short enough to need several
    verification rounds (segment-interleaved chain storage)."""
    case = deck.channel(48, 16, 500.0, 0.004, length=3.0, solver="rb_sor")
    o, met = oracle_setup(case)
    s = Solver.for_case(case)
    s.tune(seg=seg, warm=warm)
    f = fields_for(case, 21, amp=0.2)
    un, vn = f["u"], f["v"]
    o.vel_bound_cond(case.nx, case.ny, case.regions, un, vn)
    us, vs = un.copy(order="F"), vn.copy(order="F")
    gus, gvs = us.copy(order="F"), vs.copy(order="F")
    z = o.field()
    prm = case.params
    n_o = o.naux_momentum(case.nx, case.ny, case.regions, prm, met, z, z, un, vn, us, vs)
    n_g = s.nAuxMomentum(prm.mqiter, prm.dk, prm.re, prm.fr, prm.qtol, None, None, un, vn, gus, gvs)
    assert n_g == n_o
    assert np.array_equal(gus, us) and np.array_equal(gvs, vs)


@pytest.mark.parametrize("outlet", ["mc", "fd"])
def test_profiled_channel_time_loop(outlet):
    """Parabolic + perturbed inflow profile on the west face (face-profile
    extension): the device time loop bit-identical to the oracle's, with
    either outlet type."""
    case = deck.channel_inflow(96, 24, 1000.0, 0.002, seed=5, length=4.0, outlet=outlet)
    u0, v0, p0 = deck.channel_ic(case)
    ref = O.OracleRun(case, fields={"u": u0, "v": v0, "p": p0}, cold_start=False)
    ref.step(4)
    s = Solver.for_case(case)
    s.load_fields(u0, v0, p0)
    hist = s.step(case.params, 4)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in ref.history]
    u, v, p = s.store_fields()
    for name, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, ref.f[name]), (name, rel_err(g, ref.f[name]))


def _layout_cases():
    import thermal_setup

    def curvi(solver):
        def make():
            case = thermal_setup.curvilinear_case()
            case.params.npsolver = deck.PPE_SOLVERS[solver]
            case.params.msorit = 300
            return case
        return make
    return {
        "blockage_inlet_outlet": thermal_setup.blockage_case,
        "curvilinear_rb_sor": curvi("rb_sor"),
        "curvilinear_rb_lsor": curvi("rb_lsor"),
        "curvilinear_par_rb_sor": curvi("par_rb_sor"),
    }


@pytest.mark.parametrize("name", sorted(_layout_cases()))
def test_multiregion_time_loop_matches_oracle(name):
    """The device-resident loop on layouts beyond one region: an internal
    blockage with an inlet and an outlet, and a curvilinear 3 x 2 layout on
    the non-Cartesian Ppe (right-hand side re-formed before every sweep)."""
    case = _layout_cases()[name]()
    ref = O.OracleRun(case)
    ref.step(8)
    s = Solver.for_case(case, tuned=False)
    z = s.field()
    s.load_fields(z, z, z)
    assert s.cold_start(case.params) == ref.cold_nconv
    hist = s.step(case.params, 4) + s.step(case.params, 4)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in ref.history]
    for a, b in zip(hist, ref.history):
        assert a[2][:3] == b[2][:3]
    u, v, p = s.store_fields()
    for nm, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, ref.f[nm]), (nm, rel_err(g, ref.f[nm]))
    s.close()
