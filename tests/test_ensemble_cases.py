"""The batched-ensemble workload generator (CPU)."""
import numpy as np

from wolfd2_gb300 import deck


def test_ensemble_workload_draws():
    m = deck.ensemble_cases(256, seed=2024)
    assert len(m) == 256
    assert {x.n for x in m} <= set(deck.ENSEMBLE_SIZES)
    assert all(100.0 <= x.re <= 5000.0 for x in m)
    # same seed, same draws
    assert [(x.n, x.re) for x in m] == [(x.n, x.re) for x in deck.ensemble_cases(256, seed=2024)]
    for x in m[:20]:
        c = x.case
        # the unit square, h = 1/N, the drawn Re and dt = 0.5 h (capped)
        hx = np.diff(c.x[:, 0])
        assert np.allclose(hx, 1.0 / x.n, rtol=1e-12, atol=0)
        assert c.x[-1, 0] == 1.0 and c.y[0, -1] == 1.0
        assert c.nx == x.n + 1 and c.ny == x.n + 1
        assert abs(c.params.re - x.re) <= 1e-9 * x.re
        assert c.params.dk == x.dt
        assert x.dt <= x.dt_named == 0.5 / x.n
        assert x.dt / (x.re / x.n ** 2) <= 0.25 * (1 + 1e-12)


def test_partition_work_covers_and_balances():
    from wolfd2_gb300 import replicas
    m = deck.ensemble_cases(256, seed=2024)
    w = [x.case.cells for x in m]
    for world in (1, 2, 3, 8):
        parts = [replicas.partition_work(w, world, r) for r in range(world)]
        owned = sorted(i for p in parts for i in p)
        assert owned == list(range(len(w)))
        loads = [sum(w[i] for i in p) for p in parts]
        # largest-first greedy: every rank within one largest case of the mean
        assert max(loads) - min(loads) <= max(w)
