"""bench.py's multi-rank path on CPU: two gloo ranks on 127.0.0.1 split one
ensemble round-robin (no data-path collective), each advances its share
(with the CPU oracle standing in for the GPU), and the job's work is the sum
of the ranks' cells and its time the slowest rank's."""
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_partition_the_ensemble():
    mp = pytest.importorskip("torch.multiprocessing")
    import bench
    import pyoracle
    from multirank_worker import NCASES, STEPS, rank_main
    from suli_gb300._abi import PREC_FP64

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    try:
        for _ in range(2):
            r = q.get(timeout=300)
            res[r[0]] = r
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.terminate()
    assert all(p.exitcode == 0 for p in procs)
    (_, s0, c0, m0, t0, j0), (_, s1, c1, m1, t1, j1) = res[0], res[1]
    # every case of the ensemble advanced exactly once, by one rank
    assert set(s0).isdisjoint(s1)
    assert sorted(set(s0) | set(s1)) == sorted("ensemble_%d" % i for i in range(NCASES))
    # each rank's results are the case's own (the same as a serial run)
    pyoracle.Oracle.set_threads(1)
    for c in bench.ensemble_share(NCASES, 0, 1, PREC_FP64, lo=8, hi=12):
        c.params.omp_t = 0
        o, _ = bench._oracle_case(c)
        o.step(STEPS)
        got = s0.get(c.name, s1.get(c.name))
        assert got == (float(o.scalar("VOL_INS")), float(abs(o.field("W")).sum())), c.name
    assert t0 == t1 == float(c0 + c1)          # job work: the sum over ranks
    assert j0 == j1 == max(m0, m1)             # job time: the slowest rank
