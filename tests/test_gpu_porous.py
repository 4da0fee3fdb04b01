"""Porous regions on the device: the porosity division of the convective
coefficients (momentum.f:296-324, 621-649) and the PorosCoef terms of both
split steps (momentum.f:1115-1226).  The FP64 path against the oracle
(itself pinned to the translated reference on the same layouts), the mixed
step against its model (oracle/mixed.py); the bar is bit-for-bit
equality."""
import numpy as np
import pytest

import mixed as M
import oracle as O
import porous_setup
from wolfd2_gb300.gpu import PREC_MIXED, Solver

pytestmark = pytest.mark.gpu

LAYOUTS = ["row", "quad", "curvi"]


def _smooth(case, seed, amp):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 1, case.nx + 2)[:, None]
    y = np.linspace(0, 1, case.ny + 2)[None, :]
    f = np.zeros((case.nx + 2, case.ny + 2), order="F")
    for _ in range(4):
        k, l = rng.integers(1, 6, size=2)
        f += amp * rng.normal() * np.sin(k * np.pi * x + rng.uniform(0, 6)) * np.cos(l * np.pi * y)
    return f


@pytest.mark.parametrize("layout", LAYOUTS)
def test_porous_naux_momentum(layout):
    """The nAuxMomentum drop-in on a porous layout from seeded smooth
    fields: nQLiter and us, vs bit for bit."""
    case = porous_setup.case(layout)
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    s = Solver.for_case(case, tuned=False)
    un = np.asfortranarray(1.0 + _smooth(case, 3, 0.2))
    vn = np.asfortranarray(_smooth(case, 4, 0.2))
    o.vel_bound_cond(case.nx, case.ny, case.regions, un, vn)
    us, vs = un.copy(order="F"), vn.copy(order="F")
    gus, gvs = us.copy(order="F"), vs.copy(order="F")
    z = o.field()
    prm = case.params
    n_o = o.naux_momentum(case.nx, case.ny, case.regions, prm, met, z, z, un, vn, us, vs)
    n_g = s.nAuxMomentum(prm.mqiter, prm.dk, prm.re, prm.fr, prm.qtol, None, None, un, vn, gus, gvs)
    assert n_g == n_o
    assert np.array_equal(gus, us) and np.array_equal(gvs, vs)
    s.close()


@pytest.mark.parametrize("layout", LAYOUTS)
def test_porous_time_loop(layout):
    """Cold start and eight steps of the device-resident loop: iteration
    counts, norms and fields bit for bit."""
    case = porous_setup.case(layout)
    ref = O.OracleRun(case)
    ref.step(8)
    s = Solver.for_case(case, tuned=False)
    z = s.field()
    s.load_fields(z, z, z)
    assert s.cold_start(case.params) == ref.cold_nconv
    hist = s.step(case.params, 8)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in ref.history]
    for a, b in zip(hist, ref.history):
        assert a[2][:3] == b[2][:3]
    u, v, p = s.store_fields()
    for nm, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, ref.f[nm]), nm
    s.close()


UVP_REL_TOL = 1e-6  # a few mixed steps, velocity on max(|u|, |v|)
P_DYN_TOL = 4e-6    # p on max(max |p|, U^2)


@pytest.mark.parametrize("layout", LAYOUTS)
def test_porous_mixed_time_loop_matches_model(layout):
    """The mixed step on porous layouts: the FP32 momentum divides its
    ConvCoef values by the porosities and adds the PorosCoef terms in single
    precision (the tables rounded to FP32, as the oracle's single-precision
    statement rounds them); the Poisson solve takes the unit-stencil kernel
    ("quad": square cells) or the general-row one ("row": non-square cells;
    "curvi": curvilinear with cross terms).  Cold start and five steps
    bit-identical to the model, within the mixed path's tolerances of the
    FP64 oracle."""
    case = porous_setup.case(layout)
    model = M.MixedRun(case, inner=32)
    model.step(5)
    s = Solver.for_case(case, tuned=False)
    z = s.field()
    s.load_fields(z, z, z)
    assert s.cold_start(case.params, precision=PREC_MIXED, refine_sweeps=32) == model.cold_nconv
    hist = s.step(case.params, 5, precision=PREC_MIXED, refine_sweeps=32)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in model.history]
    for a, b in zip(hist, model.history):
        assert a[2][:3] == b[2][:3]
    u, v, p = s.store_fields()
    for nm, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, model.f[nm]), nm
    ref = O.OracleRun(case)
    ref.step(5)
    assert [h[1] for h in hist] == [h[1] for h in ref.history]
    scale = max(float(np.max(np.abs(ref.f["u"]))), float(np.max(np.abs(ref.f["v"]))))
    assert max(float(np.max(np.abs(u - ref.f["u"]))), float(np.max(np.abs(v - ref.f["v"])))) / scale <= UVP_REL_TOL
    assert float(np.max(np.abs(p - ref.f["p"]))) / max(float(np.max(np.abs(ref.f["p"]))), scale ** 2) <= P_DYN_TOL
    s.close()
