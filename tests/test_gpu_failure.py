"""Failure detection without a GPU fault: a device wait that nothing ends
returns the timeout status after its limit and leaves the context usable;
a run blown up to NaN is reported as the reference reports it, and the
context can be reloaded."""
import numpy as np
import pytest

from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import Solver, W2Error

pytestmark = pytest.mark.gpu

W2_E_TIMEOUT = 3


def _run(case, ic, n):
    s = Solver.for_case(case, tuned=False)
    s.load_fields(*ic)
    s.step(case.params, n)
    out = s.store_fields()
    s.close()
    return out


def test_device_wait_timeout_then_context_usable():
    case = deck.cavity(32, 100.0, 0.005, solver="rb_sor")
    ic = deck.perturbation_ic(case, 5)
    s = Solver.for_case(case, tuned=False)
    assert s.selftest_wait() == W2_E_TIMEOUT
    # the barrier state was cleared: steps on the same context are exact
    s.load_fields(*ic)
    s.step(case.params, 3)
    got = s.store_fields()
    s.close()
    for a, b in zip(got, _run(case, ic, 3)):
        assert np.array_equal(a, b)


def test_nan_blowup_reported_like_reference_then_reloadable():
    """A much too large dt drives the reference scheme to NaN; its step
    differences turn NaN (DiffMaxNorm starts from |delta(2,2)|) and its
    1e12 divergence test never fires (NaN > 1e12 is false).  The device
    reports the same records, and the context reloads and runs exactly."""
    import oracle as O
    case = deck.cavity(32, 5000.0, 0.5, solver="rb_sor")
    u, v, p = deck.perturbation_ic(case, 6, amp=0.5)
    ref = O.OracleRun(case, fields={"u": u, "v": v, "p": p}, cold_start=False)
    ref.step(6)
    s = Solver.for_case(case, tuned=False)
    s.load_fields(u, v, p)
    hist = s.step(case.params, 6)
    # the Q-L status agrees; the sweep count of a NaN Ppe does not (the
    # reference's max of |delta| skips NaN and stops at sweep 2, the
    # device's ranks NaN highest and runs to msorit; both leave NaN)
    assert [h[0] for h in hist] == [h[0] for h in ref.history]
    for h, r in zip(hist, ref.history):
        assert np.array_equal(np.array(h[2][:3]), np.array(r[2][:3]), equal_nan=True)
    assert np.isnan(hist[-1][2][0])
    got = s.store_fields()
    for a, b in zip(got, (ref.f["u"], ref.f["v"], ref.f["p"])):
        assert np.array_equal(a, b, equal_nan=True)
    ok = deck.cavity(32, 100.0, 0.005, solver="rb_sor")
    ic2 = deck.perturbation_ic(ok, 5)
    s.load_fields(*ic2)
    s.step(ok.params, 2)
    got = s.store_fields()
    s.close()
    for a, b in zip(got, _run(ok, ic2, 2)):
        assert np.array_equal(a, b)
