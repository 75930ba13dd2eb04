"""bench.py's multi-GPU path on CPU: two gloo ranks on 127.0.0.1, each
advancing its own ensemble (seed = rank) with no data-path collective; the
job's work is the sum of the ranks' cells and its time the slowest rank's."""
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_shard_the_ensemble():
    mp = pytest.importorskip("torch.multiprocessing")
    from multirank_worker import rank_main

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    try:
        for _ in range(2):
            r = q.get(timeout=120)
            res[r[0]] = r
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.terminate()
    assert all(p.exitcode == 0 for p in procs)
    (_, n0, c0, t0, m0, d0), (_, n1, c1, t1, m1, d1) = res[0], res[1]
    assert n0 != n1 and d0 != d1          # each rank has its own seeded ensemble
    assert t0 == t1 == float(c0 + c1)     # job work: the sum over ranks
    assert m0 == m1 == 11.0               # job time: the slowest rank
