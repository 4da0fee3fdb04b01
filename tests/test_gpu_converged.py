"""The time step with the Poisson solve converged: red/black SOR at the
optimal relaxation of the model problem, 2/(1 + sin(pi/n)), sor_tolerance
1e-9 and room for the sweeps it takes (the reference's own keywords
sor_relaxation, sor_tolerance, max_sor_iter).

Both precisions are checked against their CPU statements bit for bit (the
plain path against the oracle, the mixed path against oracle/mixed.py), and
both must bring the interior divergence -- dk times the Poisson residual,
reported by the device per step -- to 1e-10 or below.  The divergence of
the cells touching the boundary is dk * coefficient * (change of the frozen
ghost pressure over the step), which the reference's scheme fixes whatever
the solve does (tests/test_divergence.py); the device's report of it is
checked against the same formula."""
import numpy as np
import pytest

import mixed as M
import oracle as O
from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import PREC_MIXED, Solver

pytestmark = pytest.mark.gpu

DIV_TOL = 1e-10     # interior divergence after every converged step
VEL_TOL = 1e-5      # mixed vs plain FP64 velocity, on max(|u|, |v|)


def converged(n, sortol=1e-9):
    case = deck.cavity(n, 1000.0, 0.256 / n, solver="rb_sor")
    case.params.sorrel = float(np.float32(2.0 / (1.0 + np.sin(np.pi / n))))
    case.params.sortol = sortol
    case.params.msorit = 20000
    return case


def frozen_ghost_term(case, met, pn, p):
    nx, ny, dk = case.nx, case.ny, case.params.dk
    I, J = slice(2, nx + 1), slice(2, ny + 1)
    t = np.zeros((nx - 1, ny - 1))
    t[0, :] += dk * met["rau"][1, J] * (pn[1, J] - p[1, J])
    t[-1, :] += dk * met["rau"][nx, J] * (pn[nx + 1, J] - p[nx + 1, J])
    t[:, 0] += dk * met["rgv"][I, 1] * (pn[I, 1] - p[I, 1])
    t[:, -1] += dk * met["rgv"][I, ny] * (pn[I, ny + 1] - p[I, ny + 1])
    return t


@pytest.mark.parametrize("n", [256, 512])
def test_converged_plain_step_matches_oracle(n):
    """Plain FP64 with sorrel != 1: the generic red/black kernel at 256^2,
    the tiled two-sweeps-per-barrier kernel at 512^2."""
    case = converged(n)
    u0, v0, p0 = deck.perturbation_ic(case, 1234)
    ref = O.OracleRun(case, fields={"u": u0, "v": v0, "p": p0}, cold_start=False)
    ref.step(2)
    s = Solver.for_case(case)
    s.load_fields(u0, v0, p0)
    hist = s.step(case.params, 1)
    u1, v1, p1 = s.store_fields()
    hist += s.step(case.params, 1)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in ref.history]
    u, v, p = s.store_fields()
    for name, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, ref.f[name]), name
    nx, ny = case.nx, case.ny
    for h in hist:
        assert h[4] <= DIV_TOL, h
    div = M.divergence(nx, ny, ref.met, u, v)
    assert hist[-1][3] == float(np.max(np.abs(div)))
    assert hist[-1][4] == float(np.max(np.abs(div[1:-1, 1:-1])))
    # the boundary part is the frozen-ghost term, up to the remaining
    # Poisson residual (the size of the interior divergence)
    term = frozen_ghost_term(case, ref.met, p1, p)
    assert np.max(np.abs(div)) > 1e3 * hist[-1][4]
    assert np.max(np.abs(div - term)) <= 10.0 * hist[-1][4] + 1e-13


def test_converged_mixed_step_matches_model():
    """FP32 sweeps with FP64 refinement: bit-identical to the mixed model,
    interior divergence <= 1e-10 like the plain path, velocity within 1e-5
    of the plain FP64 solution."""
    case = converged(256)
    u0, v0, p0 = deck.perturbation_ic(case, 1234)
    inner = 128
    mref = M.MixedRun(case, fields={"u": u0, "v": v0, "p": p0}, cold_start=False, inner=inner)
    mref.step(2)
    s = Solver.for_case(case)
    s.load_fields(u0, v0, p0)
    hist = s.step(case.params, 2, precision=PREC_MIXED, refine_sweeps=inner)
    assert [(h[0], h[1]) for h in hist] == [(h[0], h[1]) for h in mref.history]
    u, v, p = s.store_fields()
    for name, g in (("u", u), ("v", v), ("p", p)):
        assert np.array_equal(g, mref.f[name]), name
    for h, hm in zip(hist, mref.history):
        assert h[3] == hm[3] and h[4] == hm[4]
        assert h[4] <= DIV_TOL, h
    s.load_fields(u0, v0, p0)
    h64 = s.step(case.params, 2)
    u64, v64, _ = s.store_fields()
    for h in h64:
        assert h[4] <= DIV_TOL, h
    scale = max(float(np.max(np.abs(u64))), float(np.max(np.abs(v64))))
    assert max(float(np.max(np.abs(u - u64))), float(np.max(np.abs(v - v64)))) <= VEL_TOL * scale
