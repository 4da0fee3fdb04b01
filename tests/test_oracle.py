"""CPU checks of the oracle against independent restatements (numpy/scipy)
and against properties the reference's discretisation must have."""
import json
import math
import os
import sys

import numpy as np
import pytest
import scipy.linalg

import oracle as O
from wolfd2_gb300 import deck

HERE = os.path.dirname(os.path.abspath(__file__))


def test_alt_trid_lu_matches_patched_banded_solve():
    """AltTridLU (momentum.f:1307-1339) divides row 1's super-diagonal by
    row 2's original diagonal.  Its L*U product is the original matrix with
    row 1's super-diagonal replaced by a3(1)*a2(1)/a2(2); solving that system
    with LAPACK must give the same x."""
    rng = np.random.default_rng(7)
    for n in (2, 3, 17, 200):
        a = np.empty((3, n))
        a[0] = rng.uniform(-0.4, 0.4, n)
        a[1] = rng.uniform(1.5, 2.5, n)
        a[2] = rng.uniform(-0.4, 0.4, n)
        b = rng.normal(size=n)
        x = O.alt_trid_lu(a, b)
        ab = np.zeros((3, n))
        ab[0, 1:] = a[2, :-1]
        ab[0, 1] = a[2, 0] * a[1, 0] / a[1, 1]
        ab[1] = a[1]
        ab[2, :-1] = a[0, 1:]
        ref = scipy.linalg.solve_banded((1, 1), ab, b)
        np.testing.assert_allclose(x, ref, rtol=1e-12, atol=1e-14)


def test_perturbation_ic_is_discretely_divergence_free():
    case = deck.cavity(48, 1000.0, 1e-3)
    u, v, p = deck.perturbation_ic(case, 3)
    nx, ny = case.nx, case.ny
    h = 1.0 / 48
    # Divergence nloc=1 on a Cartesian grid reduces to face differences
    div = (u[1:nx + 1, 1:ny + 1] - u[0:nx, 1:ny + 1]) * h + (v[1:nx + 1, 1:ny + 1] - v[1:nx + 1, 0:ny]) * h
    assert np.max(np.abs(div[1:, 1:])) < 1e-15
    assert np.max(np.abs(u)) > 0.1


def test_ppe_operator_symmetric_with_constant_nullspace():
    """The 5-point operator of pressure.f:97-106 built from the metrics:
    symmetric, and its interior rows sum to zero."""
    case = deck.channel(20, 12, 100.0, 1e-3, length=1.7)
    o = O.Oracle(case.nx + 1, case.ny + 1)
    m = o.grid(case.nx, case.ny, case.x, case.y)
    rau, rgv = m["rau"], m["rgv"]
    nx, ny = case.nx, case.ny
    for j in range(2, ny + 1):
        for i in range(2, nx + 1):
            a1, a2, a4, a5 = rgv[i, j - 1], rau[i - 1, j], rau[i, j], rgv[i, j]
            a3 = -rau[i, j] - rau[i - 1, j] - rgv[i, j] - rgv[i, j - 1]
            assert abs(a1 + a2 + a3 + a4 + a5) <= 1e-12 * abs(a3)
            if i < nx:
                assert a4 == rau[(i + 1) - 1, j]     # east coefficient = neighbour's west
            if j < ny:
                assert a5 == rgv[i, (j + 1) - 1]     # north coefficient = neighbour's south


def test_boundary_rules_on_cavity():
    case = deck.cavity(16, 100.0, 1e-3, lid=1.5)
    o = O.Oracle(case.nx + 1, case.ny + 1)
    rng = np.random.default_rng(1)
    u, v, p = (np.asfortranarray(rng.normal(size=(case.nx + 2, case.ny + 2))) for _ in range(3))
    o.vel_bound_cond(case.nx, case.ny, case.regions, u, v)
    o.pres_bound_cond(case.nx, case.ny, case.regions, p)
    nx, ny = case.nx, case.ny
    assert np.all(u[1, 1:ny + 1] == 0) and np.all(u[nx, 1:ny + 1] == 0)          # no-slip walls
    np.testing.assert_array_equal(v[1, 2:ny + 1], -v[2, 2:ny + 1])                  # image points
    np.testing.assert_array_equal(u[2:nx + 1, ny + 1], 2 * 1.5 - u[2:nx + 1, ny])   # moving lid
    np.testing.assert_array_equal(u[2:nx, 1], -u[2:nx, 2])
    np.testing.assert_array_equal(p[1, 2:ny + 1], p[2, 2:ny + 1])                   # Neumann
    np.testing.assert_array_equal(p[2:nx + 1, ny + 1], p[2:nx + 1, ny])


GOLDEN = ("cavity64_sor", "heated24_filter", "thermal_multiregion", "curvilinear_rb_lsor")


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_fixture(name):
    """The oracle's time loop reproduces each fixture of
    tests/golden/make_golden.py (generated from the translated reference
    source): iteration counts, the last step's differences, the exact
    sums and the SHA-256 of every field."""
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden
    g = json.load(open(os.path.join(HERE, "golden", name + ".json")))
    factory, steps, _, fields = make_golden.FIXTURES[name]
    assert g["steps"] == steps and g["fields"] == fields
    case = factory()
    r = O.OracleRun(case)
    r.step(g["steps"])
    keys = ("cold_nconv", "iterations", "dif_last", "sum", "abs_sum", "sha256")
    assert make_golden.summary(r, fields, case.nx, case.ny) == {k: g[k] for k in keys}


def test_face_profile_of_constants_equals_region_constant():
    """The per-position face values (an extension for inflow/lid profiles)
    reduce to the reference's region constant when every value equals it."""
    from wolfd2_gb300 import deck as D
    base = D.channel(48, 16, 500.0, 0.004, length=3.0, solver="rb_sor")
    prof = D.channel(48, 16, 500.0, 0.004, length=3.0, solver="rb_sor")
    prof.regions.profiles[(1, 1, D.WEST, 1)] = np.full(prof.ny + 2, 1.0)
    a, b = O.OracleRun(base), O.OracleRun(prof)
    a.step(3)
    b.step(3)
    assert a.history == b.history
    for n in "uvp":
        assert np.array_equal(a.f[n], b.f[n])
    lid = D.cavity(32, 100.0, 0.005, solver="rb_sor")
    run0 = O.OracleRun(lid)
    run0.step(2)
    lid.regions.profiles[(1, 1, D.NORTH, 1)] = np.full(lid.nx + 2, 1.0)
    run1 = O.OracleRun(lid)
    run1.step(2)
    assert run0.history == run1.history


def test_profiled_channel_outlet_types():
    """Profiled channel at the channel workload's CFL (dx = dy = 1/32,
    dt = 8e-3, Re = 1e4): with the mass-conserving outlet (BM_OUTLT2) the
    inflow is balanced and the divergence stays small; with the fully
    developed outlet (BM_OUTLT1) the all-Neumann pressure problem has no
    solution and the pressure change grows by a factor > 2 per step."""
    import mixed as MX
    from wolfd2_gb300 import deck as D
    res = {}
    for outlet in ("mc", "fd"):
        case = D.channel_inflow(128, 32, 1.0e4, 8.0e-3, seed=1234, outlet=outlet)
        u0, v0, p0 = D.channel_ic(case)
        r = O.OracleRun(case, fields={"u": u0, "v": v0, "p": p0}, cold_start=False)
        r.step(4)
        res[outlet] = ([h[2][0] for h in r.history],
                       MX.div_check(case.nx, case.ny, r.met, r.f["u"], r.f["v"]))
    dp, div = res["mc"]
    assert div < 1.0e-5 and dp[-1] < dp[0]
    dp, div = res["fd"]
    assert all(b > 2.0 * a for a, b in zip(dp, dp[1:])) and div > 1.0e-3
