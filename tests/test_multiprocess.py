"""N>1 paths on CPU with world_size-2 gloo ranks: independent replicas of a
single case (the reference arm's oracle on a small cavity), and the
ensemble workload's shards (the 256 drawn cavities spread by work with no
exchange), each timed and combined with the max-over-ranks reduction
bench.py uses."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    import time
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "oracle")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from wolfd2_gb300 import deck, replicas
    import oracle as O
    mine = replicas.partition(5, world, rank)
    case = deck.cavity(16, 100.0, 0.01, solver="rb_sor")
    dist.barrier()
    t0 = time.perf_counter()
    hist = []
    for k in mine:
        u, v, p = deck.perturbation_ic(case, 100 + k, modes=4)
        r = O.OracleRun(case, fields={"u": u, "v": v, "p": p}, cold_start=False)
        r.step(2)
        hist.append(r.history[-1][:2])
    dt = time.perf_counter() - t0
    (tmax,) = replicas.max_over_ranks((dt,))
    dist.barrier()
    q.put((rank, mine, hist, dt, tmax))
    dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, h0, t0, tm0), (r1, m1, h1, t1, tm1) = out
    assert m0 + m1 == [0, 1, 2, 3, 4]            # disjoint cover of the ensemble
    assert tm0 == tm1 == max(t0, t1)             # same max on every rank
    assert all(h[1] > 0 for h in h0 + h1)


def _ens_worker(rank, world, port, q):
    """One rank of the ensemble workload's N>1 path as bench.py runs it:
    the 256 drawn cavities are spread by work (cells) with
    replicas.partition_work, every rank steps its own cases with no
    exchange, and the elapsed times are reduced with max_over_ranks.  The
    CPU oracle stands in for the device (one step of the rank's two
    smallest cases, coarsened to 16 x 16 cells) so the run takes seconds."""
    import sys
    import time
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "oracle")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from wolfd2_gb300 import deck, replicas
    import oracle as O
    members = deck.ensemble_cases(256, seed=2024)
    weights = [m.case.cells for m in members]
    mine = replicas.partition_work(weights, world, rank)
    dist.barrier()
    t0 = time.perf_counter()
    counts = []
    for i in sorted(mine, key=lambda i: weights[i])[:2]:
        m = members[i]
        case = deck.cavity(16, m.re, m.dt * m.n / 16.0, solver="rb_sor")
        u, v, p = deck.perturbation_ic(case, 1234 + i, modes=4)
        r = O.OracleRun(case, fields={"u": u, "v": v, "p": p}, cold_start=False)
        r.step(1)
        counts.append(r.history[-1][:2])
    dt = time.perf_counter() - t0
    (tmax,) = replicas.max_over_ranks((dt,))
    load = sum(weights[i] for i in mine)
    dist.barrier()
    q.put((rank, mine, load, counts, dt, tmax))
    dist.destroy_process_group()


def test_two_rank_ensemble_partition_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_ens_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, l0, c0, t0, tm0), (r1, m1, l1, c1, t1, tm1) = out
    assert sorted(m0 + m1) == list(range(256)) and not set(m0) & set(m1)
    from wolfd2_gb300 import deck
    biggest = max(m.case.cells for m in deck.ensemble_cases(256, seed=2024))
    assert abs(l0 - l1) <= biggest                 # balanced to within one case
    assert tm0 == tm1 == max(t0, t1)
    assert all(c[1] > 0 for c in c0 + c1)
