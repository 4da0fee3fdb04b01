"""N>1 path on CPU: world_size-2 gloo ranks run independent replicas (the
reference arm's oracle on a small cavity), time them and combine with the
same max-over-ranks reduction bench.py uses."""
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
