"""Ensembles: many cases advanced by one launch per stage must give, per
case, exactly what the case gives when stepped alone (the same mixed or
plain step: chain solves are exact for any segment length, the Poisson
sweeps exact for any tile plan or block count)."""
import numpy as np
import pytest

from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import PREC_FP64, PREC_MIXED, Ensemble, Solver

pytestmark = pytest.mark.gpu

H = 1.0 / 64.0
REFINE = 32


def _cases():
    """Cavities of different sizes and Reynolds numbers at spacing 1/64
    (unit-stencil Poisson rows), one of them rectangular."""
    spec = [(32, None, 100.0), (48, None, 400.0), (64, None, 1000.0), (96, None, 250.0), (40, 24, 300.0)]
    out = []
    for k, (n, ny, re) in enumerate(spec):
        side = n * H
        dt = min(0.5 * H, 0.25 * H * H * re)
        case = deck.cavity(n, re, dt, solver="rb_sor", ny=ny, side=side)
        out.append((case, deck.perturbation_ic(case, 100 + k)))
    return out


def _plain_cases():
    """One case per Poisson solver, on grids the mixed step does not take:
    spacings that are not powers of two, a rectangle, and a channel with an
    outlet."""
    out = []
    spec = [(32, None, 100.0, "sor", 0.5), (40, None, 400.0, "lsor", 1.0),
            (48, 32, 300.0, "rb_lsor", 1.0), (36, None, 200.0, "par_rb_lsor", 1.0),
            (64, None, 1000.0, "rb_sor", 1.0)]
    for k, (n, ny, re, solver, side) in enumerate(spec):
        h = side / n
        dt = min(0.5 * h, 0.25 * h * h * re)
        case = deck.cavity(n, re, dt, solver=solver, ny=ny, side=side)
        out.append((case, deck.perturbation_ic(case, 200 + k)))
    ch = deck.channel_inflow(64, 16, 100.0, 0.01, solver="par_rb_sor", outlet="mc", seed=7)
    out.append((ch, deck.channel_ic(ch)))
    return out


def _alone(case, fields, nsteps, precision=PREC_MIXED):
    s = Solver.for_case(case, tuned=False)
    s.load_fields(*fields)
    hist = s.step(case.params, nsteps, precision=precision, refine_sweeps=REFINE)
    u, v, p = s.store_fields()
    s.close()
    return hist, (u, v, p)


@pytest.mark.parametrize("graph", [False, True])
def test_ensemble_matches_cases_alone(graph):
    cases = _cases()
    nsteps = 3
    solvers = []
    for case, f in cases:
        s = Solver.for_case(case, tuned=False)
        s.load_fields(*f)
        solvers.append(s)
    ens = Ensemble(solvers, graph=graph)
    hist = ens.step([c.params for c, _ in cases], nsteps, refine_sweeps=REFINE)
    info = ens.info()
    assert info["blocks_momentum"] >= len(cases) and info["blocks_poisson"] >= len(cases)
    for k, ((case, f), s) in enumerate(zip(cases, solvers)):
        ref_hist, ref = _alone(case, f, nsteps)
        assert [(h[0], h[1]) for h in hist[k]] == [(h[0], h[1]) for h in ref_hist], k
        assert [h[2][:3] for h in hist[k]] == [h[2][:3] for h in ref_hist], k
        got = s.store_fields()
        for name, g, r in zip("uvp", got, ref):
            assert np.array_equal(g, r), (k, name, float(np.max(np.abs(g - r))))
    ens.close()
    for s in solvers:
        s.close()


def test_ensemble_continues_across_calls():
    """Two calls of 2 steps equal one call of 4 (time levels carried over)."""
    cases = _cases()[:3]
    a, b = [], []
    for case, f in cases:
        for lst in (a, b):
            s = Solver.for_case(case, tuned=False)
            s.load_fields(*f)
            lst.append(s)
    ea, eb = Ensemble(a), Ensemble(b, graph=False)
    prm = [c.params for c, _ in cases]
    ea.step(prm, 2, refine_sweeps=REFINE)
    ea.step(prm, 2, refine_sweeps=REFINE)
    eb.step(prm, 4, refine_sweeps=REFINE)
    for sa, sb in zip(a, b):
        for x, y in zip(sa.store_fields(), sb.store_fields()):
            assert np.array_equal(x, y)
    ea.close()
    eb.close()
    for s in a + b:
        s.close()


@pytest.mark.parametrize("graph", [False, True])
def test_plain_ensemble_matches_cases_alone(graph):
    """The plain FP64 ensemble: every solver, non-unit grids, an outlet;
    bit-identical fields and equal iteration counts per case."""
    cases = _plain_cases()
    nsteps = 3
    solvers = []
    for case, f in cases:
        s = Solver.for_case(case, tuned=False)
        s.load_fields(*f)
        solvers.append(s)
    ens = Ensemble(solvers, graph=graph)
    hist = ens.step([c.params for c, _ in cases], nsteps, precision=PREC_FP64)
    for k, ((case, f), s) in enumerate(zip(cases, solvers)):
        ref_hist, ref = _alone(case, f, nsteps, precision=PREC_FP64)
        assert [(h[0], h[1]) for h in hist[k]] == [(h[0], h[1]) for h in ref_hist], k
        assert [h[2][:3] for h in hist[k]] == [h[2][:3] for h in ref_hist], k
        got = s.store_fields()
        for name, g, r in zip("uvp", got, ref):
            assert np.array_equal(g, r), (k, name, float(np.max(np.abs(g - r))))
    # lexicographic and line solvers have no mixed form
    with pytest.raises(Exception):
        ens.step([c.params for c, _ in cases], 1, precision=PREC_MIXED)
    ens.close()
    for s in solvers:
        s.close()


def test_ensemble_switches_precision():
    """Unit-stencil cases: plain steps then mixed steps in one ensemble equal
    the same sequence on each case alone."""
    cases = _cases()[:3]
    solvers = []
    for case, f in cases:
        s = Solver.for_case(case, tuned=False)
        s.load_fields(*f)
        solvers.append(s)
    ens = Ensemble(solvers)
    prm = [c.params for c, _ in cases]
    ens.step(prm, 2, precision=PREC_FP64)
    ens.step(prm, 2, precision=PREC_MIXED, refine_sweeps=REFINE)
    for (case, f), s in zip(cases, solvers):
        a = Solver.for_case(case, tuned=False)
        a.load_fields(*f)
        a.step(case.params, 2)
        a.step(case.params, 2, precision=PREC_MIXED, refine_sweeps=REFINE)
        for x, y in zip(s.store_fields(), a.store_fields()):
            assert np.array_equal(x, y)
        a.close()
    ens.close()
    for s in solvers:
        s.close()


def _general_cases():
    """Cases whose Poisson rows are not the unit stencil in FP32 beside
    unit-row ones: a channel with non-square cells, a blockage, a
    wall-clustered cavity, a curvilinear layout with RhsPpe's cross terms
    (lCartesGrid = 0), and two unit-row cavities."""
    import thermal_setup
    curv, _, _ = thermal_setup.problem(36, 24)
    curv.params.lcartes = 0
    gen = [deck.channel(40, 20, 800.0, 0.004, length=2.5, solver="rb_sor", outlet="mc"),
           thermal_setup.blockage_case(),
           deck.clustered_cavity(48, 400.0, 0.002, solver="rb_sor"),
           curv]
    out = [(c, deck.perturbation_ic(c, 300 + k)) for k, c in enumerate(gen)]
    return out + _cases()[:2]


@pytest.mark.parametrize("graph", [False, True])
def test_mixed_ensemble_general_rows_matches_cases_alone(graph):
    """The mixed step of an ensemble mixing general-row cases (the
    general-row Poisson kernel on their block groups) with unit-row ones
    (the multi-tile unit kernel): per case bit-identical to the case alone
    (which runs the tiled general-row form on Cartesian grids)."""
    cases = _general_cases()
    nsteps = 3
    solvers = []
    for case, f in cases:
        s = Solver.for_case(case, tuned=False)
        s.load_fields(*f)
        solvers.append(s)
    ens = Ensemble(solvers, graph=graph)
    hist = ens.step([c.params for c, _ in cases], nsteps, refine_sweeps=REFINE)
    for k, ((case, f), s) in enumerate(zip(cases, solvers)):
        ref_hist, ref = _alone(case, f, nsteps)
        assert [(h[0], h[1]) for h in hist[k]] == [(h[0], h[1]) for h in ref_hist], k
        assert [h[2][:3] for h in hist[k]] == [h[2][:3] for h in ref_hist], k
        got = s.store_fields()
        for name, g, r in zip("uvp", got, ref):
            assert np.array_equal(g, r), (k, name, float(np.max(np.abs(g - r))))
    ens.close()
    for s in solvers:
        s.close()


@pytest.mark.parametrize("precision", [PREC_MIXED, PREC_FP64])
def test_ensemble_filter_matches_cases_alone(precision):
    """Filter of us and/or vs after nAuxMomentum (utility.f:33-247, main.f:
    783-791) in some cases of an ensemble, none in others: per case
    bit-identical to the case alone."""
    cases = _cases()[:3] + [_general_cases()[1]]
    flags = [(1, 1, 4.0), (1, 0, 2.5), (0, 0, 0.0), (0, 1, 6.0)]
    for (case, _), (fu, fv, fp) in zip(cases, flags):
        case.params.nfiltu, case.params.nfiltv = fu, fv
        case.params.fpu = case.params.fpv = fp
    nsteps = 3
    solvers = []
    for case, f in cases:
        s = Solver.for_case(case, tuned=False)
        s.load_fields(*f)
        solvers.append(s)
    ens = Ensemble(solvers)
    hist = ens.step([c.params for c, _ in cases], nsteps, refine_sweeps=REFINE, precision=precision)
    for k, ((case, f), s) in enumerate(zip(cases, solvers)):
        ref_hist, ref = _alone(case, f, nsteps, precision=precision)
        assert [(h[0], h[1]) for h in hist[k]] == [(h[0], h[1]) for h in ref_hist], k
        assert [h[2][:3] for h in hist[k]] == [h[2][:3] for h in ref_hist], k
        got = s.store_fields()
        for name, g, r in zip("uvp", got, ref):
            assert np.array_equal(g, r), (k, name, float(np.max(np.abs(g - r))))
    ens.close()
    for s in solvers:
        s.close()


@pytest.mark.parametrize("precision", [PREC_MIXED, PREC_FP64])
def test_ensemble_porous_matches_cases_alone(precision):
    """Porous layouts (two regions sharing a border, three around a
    non-porous one, a curvilinear pair) beside a plain cavity in one
    ensemble: per case bit-identical to the case alone, in both
    precisions."""
    import porous_setup
    cases = [(c, deck.perturbation_ic(c, 400 + k))
             for k, c in enumerate(porous_setup.case(n) for n in ("row", "quad", "curvi"))]
    cases += _cases()[:1]
    nsteps = 3
    solvers = []
    for case, f in cases:
        s = Solver.for_case(case, tuned=False)
        s.load_fields(*f)
        solvers.append(s)
    ens = Ensemble(solvers)
    hist = ens.step([c.params for c, _ in cases], nsteps, refine_sweeps=REFINE, precision=precision)
    for k, ((case, f), s) in enumerate(zip(cases, solvers)):
        ref_hist, ref = _alone(case, f, nsteps, precision=precision)
        assert [(h[0], h[1]) for h in hist[k]] == [(h[0], h[1]) for h in ref_hist], k
        assert [h[2][:3] for h in hist[k]] == [h[2][:3] for h in ref_hist], k
        got = s.store_fields()
        for name, g, r in zip("uvp", got, ref):
            assert np.array_equal(g, r), (k, name, float(np.max(np.abs(g - r))))
    ens.close()
    for s in solvers:
        s.close()
