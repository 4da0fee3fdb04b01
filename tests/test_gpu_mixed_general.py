"""The mixed-precision Poisson solve on grids whose Poisson rows are not the
unit stencil in FP32 (oracle/mixed.py ppe_mixed_general): cells that are
not square, a Cartesian grid clustered towards the walls, blockage identity rows, and a
curvilinear grid whose right-hand side carries RhsPpe's cross terms
(lCartesGrid = 0).  The kernel evaluates every FP32 sweep and every FP64
residual/correction in the model's order and type, so against the model the
bar is bit-for-bit equality and equal sweep counts.  Against the FP64
oracle: the same sweep counts, and p within P_REL_TOL after one solve; u, v,
p within the mixed path's tolerances after time steps."""
import numpy as np
import pytest

import mixed as M
import oracle as O
import thermal_setup
from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import PREC_MIXED, Solver

pytestmark = pytest.mark.gpu

P_REL_TOL = 1e-8    # one Ppe call, mixed vs FP64 oracle
UVP_REL_TOL = 1e-6  # a few time steps, velocity on max(|u|, |v|)
P_DYN_TOL = 4e-6    # a few time steps, p on max(max |p|, U^2)


def _curvilinear(ncx=36, ncy=24):
    case, _, _ = thermal_setup.problem(ncx, ncy)
    case.params.lcartes = 0
    return case


LAYOUTS = {
    "nonsquare": lambda: deck.channel(40, 20, 800.0, 0.004, length=2.5, solver="rb_sor", outlet="mc"),
    "stretched": lambda: deck.clustered_cavity(48, 400.0, 0.002, solver="rb_sor"),
    "blockage": thermal_setup.blockage_case,
    "curvilinear": lambda: _curvilinear(),
    # grids large enough for every SM to hold blocks (the small ones run on one block)
    "nonsquare_big": lambda: deck.channel(256, 128, 800.0, 0.002, length=3.0, solver="rb_sor", outlet="mc"),
    "curvilinear_big": lambda: _curvilinear(192, 128),
}


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _inputs(case, seed, amp=0.05):
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    rng = np.random.default_rng(seed)
    u, v, p = (np.asfortranarray(rng.normal(size=(case.nx + 2, case.ny + 2)) * amp) for _ in range(3))
    o.vel_bound_cond(case.nx, case.ny, case.regions, u, v)
    o.pres_bound_cond(case.nx, case.ny, case.regions, p)
    return o, met, u, v, p


# (npsolver, sorrel, sortol, sweeps per refinement pass); the last is one
# FP32 pass over the whole solve, no refinement
SOLVES = [(5, 1.0, 1e-9, 24), (6, 1.6, 1e-8, 7), (5, 1.0, 3e-7, 5000)]
PPE_CASES = ([(lay, *sv) for lay in ("nonsquare", "stretched", "blockage", "curvilinear") for sv in SOLVES] +
             [("nonsquare_big", 5, 1.9, 1e-9, 24), ("curvilinear_big", 5, 1.9, 1e-9, 24)])


@pytest.mark.parametrize("layout,npsolver,sorrel,sortol,inner", PPE_CASES)
def test_mixed_general_ppe_matches_model(layout, npsolver, sorrel, sortol, inner):
    """Drop-in Ppe in mixed mode: bit-identical to the model.  With
    refinement passes the oracle's FP64 solve stops on the same sweep and p
    is within P_REL_TOL of it; one FP32 pass without refinement drifts from
    it (about 1e-6 of p, and a later stop), which is what the FP64 residual
    passes remove."""
    case = LAYOUTS[layout]()
    lc = case.params.lcartes
    o, met, u, v, p = _inputs(case, 23)
    s = Solver.for_case(case)
    s.set_precision(PREC_MIXED, inner)
    msorit = 3000
    gp = p.copy(order="F")
    n_g = s.Ppe(bool(lc), npsolver, msorit, case.params.dk, sortol, sorrel, u, v, gp)
    pm = p.copy(order="F")
    n_m = M.ppe_mixed_general(case.nx, case.ny, met, u, v, pm, case.params.dk, msorit, sortol, sorrel,
                              inner, regions=case.regions, lcartes=lc)
    assert n_g == n_m
    assert np.array_equal(gp, pm), _rel(gp, pm)
    prm = deck.RunParams(**{**case.params.__dict__, "sortol": sortol, "sorrel": sorrel})
    p64 = p.copy(order="F")
    n64 = o.ppe(case.nx, case.ny, case.regions, prm, met, u, v, p64, npsolver=npsolver, msorit=msorit)
    assert n64 < msorit
    if inner < n64:
        assert n_g == n64
        assert _rel(gp, p64) <= P_REL_TOL
    else:
        assert _rel(gp, p64) <= 1e-4


@pytest.mark.parametrize("layout", ["nonsquare", "stretched", "blockage", "curvilinear", "nonsquare_big"])
def test_mixed_general_time_loop_matches_model(layout):
    """Three mixed steps through wolfd2gpu_step (graph replay): the Q-L
    and sweep counts, the step norms and u, v, p bit-identical to the
    model; within the mixed path's tolerances of the FP64 oracle."""
    case = LAYOUTS[layout]()
    case.params.sortol = 1e-9
    u0, v0, p0 = deck.perturbation_ic(case, 5)
    fields = {"u": u0, "v": v0, "p": p0}
    model = M.MixedRun(case, fields=fields, cold_start=False, inner=32)
    assert model.general
    model.step(3)
    s = Solver.for_case(case)
    s.load_fields(u0, v0, p0)
    hist = s.step(case.params, 3, precision=PREC_MIXED, refine_sweeps=32)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in model.history]
    for a, b in zip(hist, model.history):
        assert a[2][:3] == b[2][:3]
    u, v, p = s.store_fields()
    for nm, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, model.f[nm]), (nm, _rel(g, model.f[nm]))
    ref = O.OracleRun(case, fields=fields, cold_start=False)
    ref.step(3)
    assert [h[1] for h in hist] == [h[1] for h in ref.history]
    scale = max(float(np.max(np.abs(ref.f["u"]))), float(np.max(np.abs(ref.f["v"]))))
    assert max(float(np.max(np.abs(u - ref.f["u"]))), float(np.max(np.abs(v - ref.f["v"])))) / scale <= UVP_REL_TOL
    assert float(np.max(np.abs(p - ref.f["p"]))) / max(float(np.max(np.abs(ref.f["p"]))), scale ** 2) <= P_DYN_TOL


def test_mixed_general_cold_start_matches_model():
    """Cold start (VelBoundCond, Ppe, PresBoundCond, Project) in mixed mode
    on the blockage layout from rest."""
    case = thermal_setup.blockage_case()
    model = M.MixedRun(case, inner=16)
    s = Solver.for_case(case)
    z = s.field()
    s.load_fields(z, z, z)
    assert s.cold_start(case.params, precision=PREC_MIXED, refine_sweeps=16) == model.cold_nconv
    u, v, p = s.store_fields()
    for nm, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, model.f[nm]), nm


@pytest.mark.parametrize("layout", ["nonsquare", "blockage", "nonsquare_big"])
@pytest.mark.parametrize("sortol,inner", [(1e-9, 24), (2e-7, 7)])
def test_mixed_general_forms_agree(layout, sortol, inner):
    """Cartesian grids run the tiled form (four sweeps per grid barrier on
    halo'd tiles) by default; the one-grid-barrier-per-colour form gives
    the same bits, and both equal the model."""
    case = LAYOUTS[layout]()
    o, met, u, v, p = _inputs(case, 31)
    out = []
    for form in (-6, -5):  # tiled, then one barrier per colour
        s = Solver.for_case(case)
        s.tune(blocks_per_sm=form)
        s.set_precision(PREC_MIXED, inner)
        gp = p.copy(order="F")
        out.append((s.Ppe(True, 5, 3000, case.params.dk, sortol, 1.0, u, v, gp), gp))
    pm = p.copy(order="F")
    n_m = M.ppe_mixed_general(case.nx, case.ny, met, u, v, pm, case.params.dk, 3000, sortol, 1.0, inner,
                              regions=case.regions)
    for n_g, gp in out:
        assert n_g == n_m
        assert np.array_equal(gp, pm), _rel(gp, pm)
