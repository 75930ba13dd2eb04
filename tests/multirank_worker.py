"""Rank body of the two-process test of bench.py's multi-rank path (runs in
a spawned child, so it lives in an importable module of its own).  Each rank
takes its round-robin share of one small ensemble, advances every case of it
with the CPU oracle (the stand-in for the GPU on a machine without one) and
reports its cases' states, its cells and the job totals."""
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

NCASES = 4
STEPS = 2


def rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        import bench
        import pyoracle
        from suli_gb300._abi import PREC_FP64

        pyoracle.Oracle.set_threads(1)
        cs = bench.ensemble_share(NCASES, rank, world, PREC_FP64, lo=8, hi=12)
        t0 = time.perf_counter()
        states = {}
        for c in cs:
            c.params.omp_t = 0            # serial CG sums: the same bits in any process
            o, _ = bench._oracle_case(c)
            o.step(STEPS)
            states[c.name] = (float(o.scalar("VOL_INS")), float(abs(o.field("W")).sum()))
        ms = (time.perf_counter() - t0) * 1e3
        cells = sum(c.cells for c in cs)
        tot, job_ms = bench.job_totals(cells, ms, dist, torch)
        out.put((rank, states, cells, ms, tot, job_ms))
    finally:
        dist.barrier()
        dist.destroy_process_group()
