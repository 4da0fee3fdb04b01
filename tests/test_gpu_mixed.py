"""GPU mixed-precision Poisson path against its CPU model (oracle/mixed.py)
and against the FP64 oracle.

The kernel evaluates every FP32 sweep and every FP64 residual/correction in
the model's order and type (no FMA contraction), so the bar against the model
is bit-for-bit equality of p and equal sweep counts, for every kernel shape.
Against the FP64 oracle the bar is the mixed path's accuracy statement: the
same sweep counts, and u, v, p within the relative tolerances below."""
import numpy as np
import pytest

import mixed as M
import oracle as O
from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import PREC_MIXED, Solver, W2Error

pytestmark = pytest.mark.gpu

P_REL_TOL = 1e-8    # one Ppe call, mixed vs FP64 oracle
UVP_REL_TOL = 1e-6  # a few time steps (FP32 momentum), mixed vs FP64 oracle: velocity
                    # on the velocity scale U = max(|u|, |v|)
P_DYN_TOL = 4e-6    # p on max(max |p|, U^2): FP32 rounding of u, v (eps32 U / h in the
                    # divergence) enters the Poisson right-hand side divided by dk, about
                    # 1e-6 U^2 on the 128x32 channel at dt = 2e-3


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _vel_rel(u, v, ru, rv):
    """Velocity error on the velocity scale: max |du|, |dv| over max |u|, |v|."""
    scale = max(float(np.max(np.abs(ru))), float(np.max(np.abs(rv))), 1e-300)
    return max(float(np.max(np.abs(u - ru))), float(np.max(np.abs(v - rv)))) / scale


def _p_rel(p, rp, ru, rv):
    """Pressure error on the dynamic-pressure scale: the FP32 momentum's
    rounding reaches p through the divergence as an absolute error of order
    eps32 * U * h / dk, whatever the size of p itself (a near-uniform channel
    flow has max |p| far below U^2)."""
    u2 = max(float(np.max(np.abs(ru))), float(np.max(np.abs(rv)))) ** 2
    return float(np.max(np.abs(p - rp))) / max(float(np.max(np.abs(rp))), u2, 1e-300)


def _inputs(case, seed, amp=0.05):
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    rng = np.random.default_rng(seed)
    u, v, p = (np.asfortranarray(rng.normal(size=(case.nx + 2, case.ny + 2)) * amp) for _ in range(3))
    o.vel_bound_cond(case.nx, case.ny, case.regions, u, v)
    o.pres_bound_cond(case.nx, case.ny, case.regions, p)
    return o, met, u, v, p


@pytest.mark.parametrize("sortol,msorit", [(1e-8, 301), (1e-8, 300), (2e-6, 2000), (7e-7, 2000),
                                           (3e-7, 2000)])
@pytest.mark.parametrize("K,threads,mode", [(8, 512, 0), (4, 256, 0), (4, 128, 0), (8, 512, 2),
                                            (4, 256, 1), (8, 256, 3), (4, 256, 3)])
def test_mixed_ppe_matches_model(sortol, msorit, K, threads, mode):
    """Drop-in Ppe in mixed mode: bit-identical to the model for stopping
    points on every sweep of a group and for odd/even msorit, with one tile
    per block (mode 0; mode 3 two such blocks per SM) and with several tiles
    per block (modes 1, 2)."""
    case = deck.cavity(128, 400.0, 0.002, solver="rb_sor", ny=64)
    o, met, u, v, p = _inputs(case, 11)
    inner = 24
    s = Solver.for_case(case)
    s.tune_mixed(K, threads, mode)
    s.set_precision(PREC_MIXED, inner)
    gp = p.copy(order="F")
    n_g = s.Ppe(True, 5, msorit, case.params.dk, sortol, case.params.sorrel, u, v, gp)
    pm = p.copy(order="F")
    n_m = M.ppe_mixed(case.nx, case.ny, met, u, v, pm, case.params.dk, msorit, sortol,
                      case.params.sorrel, inner)
    assert n_g == n_m
    assert np.array_equal(gp, pm), _rel(gp, pm)
    prm = deck.RunParams(**{**case.params.__dict__, "sortol": sortol})
    p64 = p.copy(order="F")
    n64 = o.ppe(case.nx, case.ny, case.regions, prm, met, u, v, p64, npsolver=5, msorit=msorit)
    assert n_g == n64
    assert _rel(gp, p64) <= P_REL_TOL


@pytest.mark.parametrize("sorrel", [1.25, 1.9757, 0.7])
@pytest.mark.parametrize("K,threads,mode", [(8, 512, 0), (4, 256, 1)])
def test_mixed_ppe_relaxed(sorrel, K, threads, mode):
    """Relaxation factors other than 1 (the update c + sorrel * sum rounds
    the product before the sum, pressure.f:531): bit-identical to the model
    in both tile modes."""
    case = deck.cavity(128, 400.0, 0.002, solver="rb_sor", ny=64)
    o, met, u, v, p = _inputs(case, 17)
    s = Solver.for_case(case)
    s.tune_mixed(K, threads, mode)
    s.set_precision(PREC_MIXED, 48)
    gp = p.copy(order="F")
    n_g = s.Ppe(True, 5, 700, case.params.dk, 1e-9, sorrel, u, v, gp)
    pm = p.copy(order="F")
    n_m = M.ppe_mixed(case.nx, case.ny, met, u, v, pm, case.params.dk, 700, 1e-9, sorrel, 48)
    assert n_g == n_m
    assert np.array_equal(gp, pm), _rel(gp, pm)


@pytest.mark.parametrize("inner", [1, 7, 64, 5000])
def test_mixed_ppe_refinement_lengths(inner):
    """Pass lengths that do and do not divide the group length, and one
    pass covering the whole solve."""
    case = deck.cavity(64, 100.0, 0.005, solver="rb_sor")
    o, met, u, v, p = _inputs(case, 13)
    s = Solver.for_case(case)
    s.set_precision(PREC_MIXED, inner)
    gp = p.copy(order="F")
    n_g = s.Ppe(True, 6, 400, case.params.dk, 1e-9, case.params.sorrel, u, v, gp)
    pm = p.copy(order="F")
    n_m = M.ppe_mixed(case.nx, case.ny, met, u, v, pm, case.params.dk, 400, 1e-9,
                      case.params.sorrel, inner)
    assert n_g == n_m and np.array_equal(gp, pm), _rel(gp, pm)


MIXED_CASES = {
    "cavity128": lambda: deck.cavity(128, 400.0, 0.002, solver="rb_sor"),
    "cavity_rect": lambda: deck.cavity(128, 1000.0, 0.001, solver="rb_sor", ny=32),
}


@pytest.mark.parametrize("name", sorted(MIXED_CASES))
def test_mixed_time_loop_matches_model(name):
    case = MIXED_CASES[name]()
    u0, v0, p0 = deck.perturbation_ic(case, 99)
    fields = {"u": u0, "v": v0, "p": p0}
    model = M.MixedRun(case, fields=fields, cold_start=False, inner=32)
    model.step(3)
    s = Solver.for_case(case)
    s.load_fields(u0, v0, p0)
    hist = s.step(case.params, 3, precision=PREC_MIXED, refine_sweeps=32)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in model.history]
    for a, b in zip(hist, model.history):
        assert a[2][:3] == b[2][:3]
        assert a[3] == b[3]  # divergence check
    u, v, p = s.store_fields()
    for nm, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, model.f[nm]), (nm, _rel(g, model.f[nm]))
    ref = O.OracleRun(case, fields=fields, cold_start=False)
    ref.step(3)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in ref.history]
    assert _vel_rel(u, v, ref.f["u"], ref.f["v"]) <= UVP_REL_TOL
    assert _p_rel(p, ref.f["p"], ref.f["u"], ref.f["v"]) <= P_DYN_TOL


def test_mixed_cold_start_matches_model():
    case = deck.cavity(64, 100.0, 0.005, solver="rb_sor")
    model = M.MixedRun(case, inner=16)
    s = Solver.for_case(case)
    z = s.field()
    s.load_fields(z, z, z)
    assert s.cold_start(case.params, precision=PREC_MIXED, refine_sweeps=16) == model.cold_nconv
    u, v, p = s.store_fields()
    for nm, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, model.f[nm]), nm


def test_plain_path_divergence_check():
    """The FP64 path reports max |Divergence| of its projected field."""
    case = deck.cavity(64, 100.0, 0.005, solver="rb_sor")
    ref = O.OracleRun(case)
    ref.step(2)
    s = Solver.for_case(case)
    z = s.field()
    s.load_fields(z, z, z)
    s.cold_start(case.params)
    hist = s.step(case.params, 2)
    assert hist[-1][3] == M.div_check(case.nx, case.ny, ref.met, ref.f["u"], ref.f["v"])


def test_mixed_rejects_unsupported():
    case = deck.cavity(64, 100.0, 0.005, solver="sor")
    s = Solver.for_case(case)
    z = s.field()
    s.load_fields(z, z, z)
    with pytest.raises(W2Error):
        s.step(case.params, 1, precision=PREC_MIXED)  # lexicographic SOR
    with pytest.raises(W2Error):
        s.tune_mixed(2, 0)


@pytest.mark.parametrize("n", [48, 96])
def test_mixed_non_dyadic_grid_matches_model(n):
    """h = 1/n with n not a power of two: the Poisson rows miss the unit
    stencil by rounding in FP64 but round to it in FP32, so the FP32 sweeps
    run the unit stencil and every pass's FP64 residual the grid's own
    rows.  Bit-identical to the model, close to the FP64 oracle."""
    case = deck.cavity(n, 400.0, 0.25 / n, solver="rb_sor")
    u0, v0, p0 = deck.perturbation_ic(case, 3)
    fields = {"u": u0, "v": v0, "p": p0}
    model = M.MixedRun(case, fields=fields, cold_start=False, inner=32)
    model.step(3)
    s = Solver.for_case(case)
    s.load_fields(u0, v0, p0)
    hist = s.step(case.params, 3, precision=PREC_MIXED, refine_sweeps=32)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in model.history]
    u, v, p = s.store_fields()
    for nm, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, model.f[nm]), (nm, _rel(g, model.f[nm]))
    ref = O.OracleRun(case, fields=fields, cold_start=False)
    ref.step(3)
    assert [h[1] for h in hist] == [h[1] for h in ref.history]
    assert _vel_rel(u, v, ref.f["u"], ref.f["v"]) <= UVP_REL_TOL
    assert _p_rel(p, ref.f["p"], ref.f["u"], ref.f["v"]) <= P_DYN_TOL


@pytest.mark.parametrize("tma", [True, False])
def test_mixed_multitile_time_loop_matches_model(tma):
    """Several tiles per block (16 blocks on a 256x256 cavity), the boxes
    staged by TMA tensor copies or by vector loads: the time loop
    bit-identical to the model."""
    case = deck.cavity(256, 1000.0, 0.001, solver="rb_sor")
    u0, v0, p0 = deck.perturbation_ic(case, 7)
    model = M.MixedRun(case, fields={"u": u0, "v": v0, "p": p0}, cold_start=False, inner=48)
    model.step(2)
    s = Solver.for_case(case)
    s.set_tma(tma)
    s.tune_mixed(8, 512, 2)
    s.load_fields(u0, v0, p0)
    hist = s.step(case.params, 2, precision=PREC_MIXED, refine_sweeps=48)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in model.history]
    u, v, p = s.store_fields()
    for nm, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, model.f[nm]), (nm, _rel(g, model.f[nm]))


def test_mixed_profiled_channel_matches_model():
    """Mixed path on the profiled channel (inflow profile, mass-conserving
    outlet): bit-identical to the model, close to the FP64 oracle."""
    case = deck.channel_inflow(128, 32, 1000.0, 0.002, seed=5, length=4.0)
    u0, v0, p0 = deck.channel_ic(case)
    fields = {"u": u0, "v": v0, "p": p0}
    model = M.MixedRun(case, fields=fields, cold_start=False, inner=32)
    model.step(3)
    s = Solver.for_case(case)
    s.load_fields(u0, v0, p0)
    hist = s.step(case.params, 3, precision=PREC_MIXED, refine_sweeps=32)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in model.history]
    u, v, p = s.store_fields()
    for nm, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, model.f[nm]), (nm, _rel(g, model.f[nm]))
    ref = O.OracleRun(case, fields=fields, cold_start=False)
    ref.step(3)
    assert _vel_rel(u, v, ref.f["u"], ref.f["v"]) <= UVP_REL_TOL
    assert _p_rel(p, ref.f["p"], ref.f["u"], ref.f["v"]) <= P_DYN_TOL
