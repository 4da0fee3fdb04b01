"""The oracle pinned to the reference's own source: a mechanical Fortran-77
-> C translation of src/momentum.f, src/pressure.f, src/utility.f,
src/bound_cond.f and src/grid.f (oracle/f77ref.py), sequenced as in
src/main.f (oracle/refrun.py), must give bit-identical fields and identical
iteration counts.  Skipped where neither the reference tree nor a previously
generated translation is present."""
import numpy as np
import pytest

import f77ref
import oracle as O
from wolfd2_gb300 import deck

if not (f77ref.available() or f77ref.build() is not None):
    pytest.skip("reference translation unavailable", allow_module_level=True)

import refrun  # noqa: E402

CASES = [
    ("cavity32_sor", lambda: deck.cavity(32, 100.0, 0.005, solver="sor")),
    ("cavity32_rb_sor", lambda: deck.cavity(32, 100.0, 0.005, solver="rb_sor")),
    ("cavity32_par_rb_sor", lambda: deck.cavity(32, 400.0, 0.004, solver="par_rb_sor")),
    ("rect_lsor", lambda: deck.cavity(40, 400.0, 0.004, solver="lsor", ny=24)),
    ("rect_rb_lsor", lambda: deck.cavity(36, 250.0, 0.004, solver="rb_lsor", ny=28)),
    ("channel_par_rb_lsor", lambda: deck.channel(48, 16, 500.0, 0.004, length=3.0, solver="par_rb_lsor")),
    ("channel_rb_sor", lambda: deck.channel(40, 20, 800.0, 0.003, length=2.0, solver="rb_sor")),
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_time_loop_bitwise(name, make):
    case = make()
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case)
    o = O.OracleRun(case)
    assert r.cold_nconv == o.cold_nconv
    for k in "uvp":
        assert np.array_equal(r.f[k], o.f[k]), f"cold start {k}"
    r.step(10)
    o.step(10)
    assert [h[:2] for h in r.history] == [h[:2] for h in o.history]
    for a, b in zip(r.history, o.history):
        assert a[2] == b[2]
    for k in "uvp":
        assert np.array_equal(r.f[k], o.f[k]), k


def test_blockage_and_porous_free_multiregion():
    """Three regions in i with an internal blockage and an outlet: exercises
    the blockage rows of Ppe/momentum and the region loops of the BCs."""
    text = ("number_of_regions 3 1\n i_borders 12 20\n j_borders\n"
            "blockage 2 1\n inlet 1 1 west nv 1.0\n outlet 3 1 east fd\n")
    case = deck.channel(32, 14, 300.0, 0.003, length=2.0, solver="rb_sor")
    case.regions = deck.parse_bc_section(text, case.nx, case.ny, re=case.params.re)
    case.bc_text = text
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case)
    o = O.OracleRun(case)
    r.step(6)
    o.step(6)
    assert [h[:2] for h in r.history] == [h[:2] for h in o.history]
    for k in "uvp":
        assert np.array_equal(r.f[k], o.f[k]), k


def test_named_dt_diverges_at_1024():
    """At 1024x1024, Re=1000 the named dt=1e-3 drives the reference's own
    Newton-Kantorovich iteration to NaN in the first step (both in the
    translation and in the oracle); dt=2.5e-4 stays finite."""
    case = deck.cavity(1024, 1000.0, 1e-3, solver="rb_sor")
    u, v, p = deck.perturbation_ic(case, 1234)
    f77ref.build(case.nx + 1, case.ny + 1)
    r = refrun.RefRun(case, fields={"u": u, "v": v, "p": p}, cold_start=False)
    h = r.step(1)
    assert h[0] == -1 and not np.isfinite(r.f["u"]).all()
