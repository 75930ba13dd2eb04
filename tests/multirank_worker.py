"""Rank body of the two-process test of bench.py's weak-scaling path (runs
in a spawned child, so it lives in an importable module of its own)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


class _Args:
    workload = "ensemble"
    ncases = 3
    precond = "multigrid"


def rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        import bench
        from suli_gb300._abi import PREC_MIXED

        name, cs = bench.make_cases(_Args, PREC_MIXED, rank)
        cells = sum(c.cells for c in cs)
        # each rank reports its own time; the job takes the slowest
        tot, ms = bench.job_totals(cells, 10.0 + rank, dist, torch)
        out.put((rank, name, cells, tot, ms, [list(c.params.nx for c in cs)]))
    finally:
        dist.barrier()
        dist.destroy_process_group()
