"""Snapshots streamed from the device: a copy of the current time level
queued on the copy stream while later steps run must hold exactly that
level, and the step that overwrites the level must wait for it (the run
itself stays bit-identical to one without snapshots)."""
import numpy as np
import pytest

from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import Solver

pytestmark = pytest.mark.gpu


def _pinned(s, n):
    import torch
    return [torch.zeros((s.mny + 1, s.mnx + 1), dtype=torch.float64, pin_memory=True).numpy().T
            for _ in range(n)]


@pytest.mark.parametrize("thermal", [False, True])
def test_snapshot_overlaps_steps(thermal):
    if thermal:
        case = deck.heated_cavity(64, 400.0, 0.004, nmeiter=2, dmeittol=0.0)
    else:
        case = deck.cavity(64, 400.0, 0.004, solver="rb_sor")
    ic = deck.perturbation_ic(case, 21)
    t0 = np.zeros_like(ic[0]) + 0.5

    def solver():
        s = Solver.for_case(case, tuned=False)
        s.load_fields(*ic)
        if thermal:
            s.load_thermal(np.asfortranarray(t0))
        return s

    # reference levels, without snapshots
    r = solver()
    r.step(case.params, 1)
    ref1 = r.store_fields() + ((r.store_thermal()[0],) if thermal else ())
    r.step(case.params, 3)
    ref4 = r.store_fields() + ((r.store_thermal()[0],) if thermal else ())
    r.close()

    s = solver()
    s.step(case.params, 1)
    host = _pinned(s, 4 if thermal else 3)
    s.snapshot(host)
    s.step(case.params, 1)   # writes the other level: runs beside the copy
    s.step(case.params, 2)   # overwrites the snapshot's level: waits for it
    s.snapshot_wait()
    for a, b in zip(host, ref1):
        assert np.array_equal(a, b)
    got4 = s.store_fields() + ((s.store_thermal()[0],) if thermal else ())
    for a, b in zip(got4, ref4):
        assert np.array_equal(a, b)
    # a snapshot written out in the reference's Plot3D solution layout
    s.snapshot(host)
    s.snapshot_wait()
    s.close()


def test_step_log(tmp_path):
    """The per-step JSONL log carries PrintDiff's fields, one line a step."""
    import json
    case = deck.cavity(32, 100.0, 0.005, solver="rb_sor")
    s = Solver.for_case(case, tuned=False)
    s.load_fields(*deck.perturbation_ic(case, 3))
    path = str(tmp_path / "steps.jsonl")
    hist = s.step_log(case.params, 3, path, k0=10, dtime0=1.0)
    s.close()
    recs = [json.loads(x) for x in open(path)]
    assert [r["k"] for r in recs] == [11, 12, 13]
    assert [(r["nQLiter"], r["nSorConv"]) for r in recs] == [(h[0], h[1]) for h in hist]
    assert recs[-1]["time"] == pytest.approx(1.0 + 3 * case.params.dk)
    assert len(recs[0]["dif"]) == 4
