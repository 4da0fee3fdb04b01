"""The device time loop against the golden fixtures of tests/golden (made
from the translated reference source), with no oracle in the loop: zero
fields, cold start, then the fixture's steps through the C-ABI; iteration
counts, the last step's differences, the exact sums and the SHA-256 of
every field must equal the fixture's.  The 64x64 cavity fixture is the
whole 500-step run of that configuration (lexicographic point SOR)."""
import json
import os
import sys

import pytest

from wolfd2_gb300.gpu import Solver

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu


class _Run:
    """The device fields in the shape make_golden.summary reads."""

    def __init__(self, cold_nconv, history, f):
        self.cold_nconv, self.history, self.f = cold_nconv, history, f


@pytest.mark.parametrize("name", sorted(make_golden.FIXTURES))
def test_device_matches_golden(name):
    g = json.load(open(os.path.join(HERE, "golden", name + ".json")))
    factory, steps, _, fields = make_golden.FIXTURES[name]
    case = factory()
    s = Solver.for_case(case, tuned=False)
    z = s.field()
    s.load_fields(z, z, z)
    nconv = s.cold_start(case.params)
    hist = s.step(case.params, steps)
    u, v, p = s.store_fields()
    f = {"u": u, "v": v, "p": p}
    if "t" in fields:
        f["t"], f["d"] = s.store_thermal()
    s.close()
    got = make_golden.summary(_Run(nconv, [(h[0], h[1], tuple(h[2])) for h in hist], f), fields,
                              case.nx, case.ny)
    for k in ("cold_nconv", "iterations", "dif_last", "sum", "abs_sum", "sha256"):
        assert got[k] == g[k], (name, k, got[k], g[k])
