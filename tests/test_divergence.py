"""The divergence of the projected field, on the CPU oracle.

With the Poisson iteration converged (red/black SOR at near-optimal
relaxation and a tight sor_tolerance, all through the reference's own
input keywords), the divergence splits in two:

* interior cells (i, j = 3..n-1: every neighbour a Poisson unknown, every
  face updated by Project): dk times the Poisson residual, which the solve
  drives below 1e-10;
* cells touching the boundary: dk * coefficient * (ghost pressure before
  the step - ghost pressure after it) on each boundary face.  Ppe solves
  with the ghost values PresBoundCond set before the call and keeps them
  frozen (src/main.f:793-811, src/pressure.f:86-87), Project then uses the
  interior pressures only (src/utility.f:299-306), and PresBoundCond moves
  the ghosts afterwards; so this part is set by how much the pressure
  changes over the step, not by the solver's tolerance or precision.

The CUDA path reports both maxima per step (w2_stepstat divmax and
divmax_int); these tests pin the split on the oracle itself."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

import mixed as M  # noqa: E402
import oracle as O  # noqa: E402
from wolfd2_gb300 import deck  # noqa: E402


def converged_cavity(n, sortol=1e-12, solver="rb_sor"):
    """Lid-driven cavity, Re 1000, CFL dt*n = 0.256 as in the 1024x1024
    benchmark, red/black SOR at the optimal relaxation of the model
    problem, 2/(1 + sin(pi/n)), and a tight tolerance."""
    case = deck.cavity(n, 1000.0, 0.256 / n, solver=solver)
    case.params.sorrel = 2.0 / (1.0 + np.sin(np.pi / n))
    case.params.sortol = sortol
    case.params.msorit = 100000
    return case


def frozen_ghost_term(case, met, f):
    """dk * coefficient * (pn - p) at the ghost of every boundary face,
    summed per pressure cell: the divergence the frozen ghosts leave."""
    nx, ny, dk = case.nx, case.ny, case.params.dk
    I, J = slice(2, nx + 1), slice(2, ny + 1)
    pn, p = f["pn"], f["p"]
    t = np.zeros((nx - 1, ny - 1))
    t[0, :] += dk * met["rau"][1, J] * (pn[1, J] - p[1, J])
    t[-1, :] += dk * met["rau"][nx, J] * (pn[nx + 1, J] - p[nx + 1, J])
    t[:, 0] += dk * met["rgv"][I, 1] * (pn[I, 1] - p[I, 1])
    t[:, -1] += dk * met["rgv"][I, ny] * (pn[I, ny + 1] - p[I, ny + 1])
    return t


def test_boundary_divergence_is_the_frozen_ghost_change():
    case = converged_cavity(64)
    u, v, p = deck.perturbation_ic(case, 1234)
    r = O.OracleRun(case, {"u": u, "v": v, "p": p}, cold_start=False)
    r.step(3)
    div = M.divergence(case.nx, case.ny, r.met, r.f["u"], r.f["v"])
    term = frozen_ghost_term(case, r.met, r.f)
    assert np.max(np.abs(div)) > 1e-5                      # a real, non-zero boundary part
    assert np.max(np.abs(div[1:-1, 1:-1])) <= 1e-12       # interior: converged to rounding
    assert np.max(np.abs(div - term)) <= 1e-12 * max(1.0, np.max(np.abs(div)))


@pytest.mark.parametrize("sortol", [1e-7, 1e-9, 1e-11])
def test_interior_divergence_follows_the_tolerance(sortol):
    """The interior divergence falls with sor_tolerance, the boundary part
    does not move."""
    case = converged_cavity(64, sortol)
    u, v, p = deck.perturbation_ic(case, 1234)
    r = O.OracleRun(case, {"u": u, "v": v, "p": p}, cold_start=False)
    r.step(2)
    div = M.divergence(case.nx, case.ny, r.met, r.f["u"], r.f["v"])
    inner = float(np.max(np.abs(div[1:-1, 1:-1])))
    assert inner <= 0.1 * sortol
    assert np.max(np.abs(div - frozen_ghost_term(case, r.met, r.f))) <= 0.1 * sortol + 1e-13


def test_mixed_model_reaches_the_same_interior_divergence():
    """FP32 sweeps with FP64 residual and correction converge the interior
    divergence as far as the plain FP64 solve (the refinement recovers what
    FP32 rounding alone could not), at the same sweep counts up to a few."""
    case = converged_cavity(64, 1e-11)
    u, v, p = deck.perturbation_ic(case, 7)
    r = O.OracleRun(case, {"u": u, "v": v, "p": p}, cold_start=False)
    mx = M.MixedRun(case, {"u": u, "v": v, "p": p}, cold_start=False, inner=64)
    r.step(3)
    mx.step(3)
    for h64, h32 in zip(r.history, mx.history):
        assert abs(h64[1] - h32[1]) <= 8, (h64[:2], h32[:2])
    d64 = M.div_check_interior(case.nx, case.ny, r.met, r.f["u"], r.f["v"])
    assert mx.history[-1][4] <= 1e-10 and d64 <= 1e-10
    # FP32 sweeps without refinement stall far above that
    case1 = converged_cavity(64, 1e-11)
    case1.params.msorit = 3000
    m1 = M.MixedRun(case1, {"u": u, "v": v, "p": p}, cold_start=False, inner=10 ** 9)
    m1.step(1)
    assert m1.history[-1][4] > 1e3 * mx.history[0][4]
