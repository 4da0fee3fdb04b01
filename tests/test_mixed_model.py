"""The mixed-precision Ppe model (FP32 red/black sweeps on the correction
equation, FP64 residual and correction) against the FP64 oracle: the same
sweep count at every stopping point, and p within the stated tolerance.
CPU only; the GPU kernel is held to this model bit for bit in
test_gpu_mixed.py."""
import numpy as np
import pytest

import mixed as M
import oracle as O
from wolfd2_gb300 import deck

# p after a mixed solve differs from the FP64 solve by FP32 rounding of one
# refinement pass's correction at most: 1e-8 of max|p| at these sizes.
P_REL_TOL = 1e-8


def _setup(n=64, seed=3):
    case = deck.cavity(n, 100.0, 0.005, solver="rb_sor")
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    rng = np.random.default_rng(seed)
    f = [np.asfortranarray(rng.normal(size=(case.nx + 2, case.ny + 2)) * 0.05) for _ in range(3)]
    u, v, p = f
    o.vel_bound_cond(case.nx, case.ny, case.regions, u, v)
    o.pres_bound_cond(case.nx, case.ny, case.regions, p)
    return case, o, met, u, v, p


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("sortol", [1e-6, 1e-7, 3e-8])
@pytest.mark.parametrize("inner", [8, 64])
def test_mixed_model_stops_where_fp64_stops(sortol, inner):
    case, o, met, u, v, p = _setup()
    prm = deck.RunParams(**{**case.params.__dict__, "sortol": sortol})
    p64 = p.copy(order="F")
    n64 = o.ppe(case.nx, case.ny, case.regions, prm, met, u, v, p64, npsolver=5, msorit=4000)
    pm = p.copy(order="F")
    nm = M.ppe_mixed(case.nx, case.ny, met, u, v, pm, prm.dk, 4000, sortol, prm.sorrel, inner)
    assert n64 < 4000 and nm == n64
    assert _rel(pm, p64) <= P_REL_TOL


def test_mixed_model_fp64_sweeps_equal_plain_solve():
    """With FP64 sweeps the refinement form is the plain iteration up to
    rounding: the algebra of the correction equation is right."""
    case, o, met, u, v, p = _setup(32, seed=5)
    prm = case.params
    p64 = p.copy(order="F")
    n64 = o.ppe(case.nx, case.ny, case.regions, prm, met, u, v, p64, npsolver=5, msorit=500)
    pm = p.copy(order="F")
    nm = M.ppe_mixed(case.nx, case.ny, met, u, v, pm, prm.dk, 500, prm.sortol, prm.sorrel, 37,
                     dtype=np.float64)
    assert nm == n64
    assert _rel(pm, p64) <= 1e-13


def test_divergence_matches_oracle_rhs():
    """The model's divergence is the oracle's b*dk on the pressure cells."""
    case, o, met, u, v, p = _setup(32, seed=7)
    div = M.divergence(case.nx, case.ny, met, u, v)
    # one FP64 sweep from p = b-consistent start: compare through the oracle's
    # Ppe with msorit = 1 on the unit stencil: p_new - p_old = sum
    p1 = p.copy(order="F")
    o.ppe(case.nx, case.ny, case.regions, case.params, met, u, v, p1, npsolver=5, msorit=1)
    # black points of the first sweep see only old neighbours
    b = div / case.params.dk
    i, j = 2, 2  # (i+j) even: black
    s = b[i - 2, j - 2] - p[i, j - 1] - p[i - 1, j] - p[i + 1, j] - p[i, j + 1]
    s = s / -4.0 - p[i, j]
    assert p1[i, j] == p[i, j] + 1.0 * s


def test_fp32_momentum_close_to_fp64():
    """The oracle's single-precision nAuxMomentum against its FP64 instance:
    the same Q-L count and us, vs within 1e-6 relative."""
    case = deck.cavity(64, 400.0, 0.004, solver="rb_sor")
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    u0, v0, _ = deck.perturbation_ic(case, 5)
    u0, v0 = u0.copy(order="F"), v0.copy(order="F")
    o.vel_bound_cond(case.nx, case.ny, case.regions, u0, v0)
    us, vs, z = u0.copy(order="F"), v0.copy(order="F"), o.field()
    n64 = o.naux_momentum(case.nx, case.ny, case.regions, case.params, met, z, z, u0, v0, us, vs)
    un32, vn32 = (np.asfortranarray(a.astype(np.float32)) for a in (u0, v0))
    us32, vs32, z32 = un32.copy(order="F"), vn32.copy(order="F"), o.field32()
    n32 = o.naux_momentum_f32(case.nx, case.ny, case.regions, case.params, o.metrics32(met),
                              z32, z32, un32, vn32, us32, vs32)
    assert n32 == n64 > 0
    assert _rel(us32.astype(np.float64), us) <= 1e-6
    assert _rel(vs32.astype(np.float64), vs) <= 1e-6


def test_mixed_time_loop_close_to_fp64():
    """A few steps of the 64x64 cavity: mixed (FP32 momentum, mixed Ppe) vs
    the FP64 oracle, u, v, p within 1e-6 relative, same iteration counts,
    the divergence check of the same size as the FP64 path's."""
    case = deck.cavity(64, 100.0, 0.005, solver="rb_sor")
    ref = O.OracleRun(case)
    ref.step(4)
    mx = M.MixedRun(case, inner=32)
    mx.step(4)
    assert mx.cold_nconv == ref.cold_nconv
    assert [(h[0], h[1]) for h in mx.history] == [(h[0], h[1]) for h in ref.history]
    for name in "uvp":
        assert _rel(mx.f[name], ref.f[name]) <= 1e-6, name
    d64 = M.div_check(case.nx, case.ny, ref.met, ref.f["u"], ref.f["v"])
    assert mx.history[-1][3] <= 2.0 * d64 + 1e-14


def _general_layouts():
    import thermal_setup
    case_c, _, _ = thermal_setup.problem()
    case_c.params.lcartes = 0
    st = deck.cavity(40, 400.0, 0.001, solver="rb_sor")
    st.x = 0.5 * (1.0 - np.cos(np.pi * st.x))
    st.y = 0.5 * (1.0 - np.cos(np.pi * st.y))
    return {"nonsquare": deck.channel(40, 20, 800.0, 0.004, length=2.5, solver="rb_sor", outlet="mc"),
            "stretched": st, "blockage": thermal_setup.blockage_case(), "curvilinear": case_c}


@pytest.mark.parametrize("sorrel", [1.0, 1.7])
def test_general_model_equals_unit_model_on_unit_rows(sorrel):
    """On unit rows every operation of the general-row sweep rounds as the
    unit form's (1 x == x, x / -4 == x * -0.25): the same p bit for bit."""
    case, o, met, u, v, p = _setup(48, seed=9)
    p1, p2 = p.copy(order="F"), p.copy(order="F")
    n1 = M.ppe_mixed(case.nx, case.ny, met, u, v, p1, case.params.dk, 500, 1e-7, sorrel, 32)
    n2 = M.ppe_mixed_general(case.nx, case.ny, met, u, v, p2, case.params.dk, 500, 1e-7, sorrel, 32,
                             regions=case.regions)
    assert n1 == n2 and np.array_equal(p1, p2)


@pytest.mark.parametrize("layout", ["nonsquare", "stretched", "blockage", "curvilinear"])
@pytest.mark.parametrize("sortol", [1e-6, 1e-9])
def test_general_model_stops_where_fp64_stops(layout, sortol):
    """General rows (non-square and unequal cells, blockage identity rows,
    RhsPpe's cross terms on a curvilinear grid): the FP32 sweeps with FP64
    refinement stop on the oracle's sweep and land within P_REL_TOL of its
    p; at the tight tolerance the two agree to 1e-12."""
    case = _general_layouts()[layout]
    o = O.Oracle(case.nx + 1, case.ny + 1)
    met = o.grid(case.nx, case.ny, case.x, case.y)
    rng = np.random.default_rng(2)
    u, v, p = (np.asfortranarray(rng.normal(size=(case.nx + 2, case.ny + 2)) * 0.05) for _ in range(3))
    o.vel_bound_cond(case.nx, case.ny, case.regions, u, v)
    o.pres_bound_cond(case.nx, case.ny, case.regions, p)
    assert not (case.params.lcartes and M.is_unit_stencil32(case.nx, case.ny, met)
                and not M.blockage_rows(case.nx, case.ny, case.regions).any())
    prm = deck.RunParams(**{**case.params.__dict__, "sortol": sortol})
    p64 = p.copy(order="F")
    n64 = o.ppe(case.nx, case.ny, case.regions, prm, met, u, v, p64, npsolver=5, msorit=3000)
    pm = p.copy(order="F")
    nm = M.ppe_mixed_general(case.nx, case.ny, met, u, v, pm, prm.dk, 3000, sortol, prm.sorrel, 32,
                             regions=case.regions, lcartes=prm.lcartes)
    assert n64 < 3000 and nm == n64
    assert _rel(pm, p64) <= (1e-12 if sortol < 1e-8 else P_REL_TOL)


@pytest.mark.parametrize("layout", ["nonsquare", "blockage", "curvilinear"])
def test_general_model_time_loop_close_to_fp64(layout):
    """The mixed time loop with general Poisson rows (FP32 momentum, general
    FP32 sweeps with FP64 refinement): the oracle's Q-L and sweep counts
    over three steps, velocity within 1e-6 of the FP64 oracle."""
    case = _general_layouts()[layout]
    case.params.sortol = 1e-9
    u0, v0, p0 = deck.perturbation_ic(case, 5)
    fields = {"u": u0, "v": v0, "p": p0}
    mx = M.MixedRun(case, fields=fields, cold_start=False, inner=32)
    assert mx.general
    mx.step(3)
    ref = O.OracleRun(case, fields=fields, cold_start=False)
    ref.step(3)
    assert [h[:2] for h in mx.history] == [h[:2] for h in ref.history]
    scale = max(float(np.max(np.abs(ref.f["u"]))), float(np.max(np.abs(ref.f["v"]))))
    err = max(float(np.max(np.abs(mx.f["u"] - ref.f["u"]))), float(np.max(np.abs(mx.f["v"] - ref.f["v"]))))
    assert err / scale <= 1e-6
