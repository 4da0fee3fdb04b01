"""CUDA-graph replay of wolfd2gpu_step against direct launches: the same
bits, through cache hits (both time-level parities, repeated calls) and
misses (a re-tuned device view, changed parameters, another step count)."""
import dataclasses

import numpy as np
import pytest

from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import PREC_FP64, PREC_MIXED, Solver

pytestmark = pytest.mark.gpu


def _run(case, fields, graph):
    s = Solver.for_case(case, tuned=False)
    s.graph(graph)
    s.load_fields(*fields)
    hist = []
    for prec in (PREC_FP64, PREC_MIXED):
        for _ in range(3):
            hist += s.step(case.params, 1, precision=prec, refine_sweeps=32)
        hist += s.step(case.params, 2, precision=prec, refine_sweeps=32)
    s.tune(seg=16)
    hist += s.step(case.params, 2)
    hist += s.step(dataclasses.replace(case.params, dk=case.params.dk * 0.5), 1)
    hist += s.step(case.params, 1, precision=PREC_MIXED, refine_sweeps=32)
    out = (hist, s.store_fields(), s.launch_count())
    s.close()
    return out


@pytest.mark.parametrize("n", [64, 128])
def test_graph_replay_matches_direct_launches(n):
    case = deck.cavity(n, 400.0, 0.002, solver="rb_sor")
    f = deck.perturbation_ic(case, 3)
    hg, fg, lg = _run(case, f, True)
    hd, fd, ld = _run(case, f, False)
    assert [(h[0], h[1], h[2][:3]) for h in hg] == [(h[0], h[1], h[2][:3]) for h in hd]
    for a, b in zip(fg, fd):
        assert np.array_equal(a, b)
    # the replayed launches are counted like direct ones
    assert lg == ld
