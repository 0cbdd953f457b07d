"""The multi-rank path of bench.py on the host (gloo, world size 2): every rank solves its own
replica, the job's time is the slowest rank's (a MAX all-reduce), and the reported value is
that time per solve of all replicas. No GPU and no collective on the solve path itself."""
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import sys

    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    local = [3.0, 5.0][rank]  # seconds this rank's replica took for its steps
    t = bench.max_over_ranks(local, ws, device="cpu")
    out.put((rank, t, bench.aggregate_per_solve(t, ws, 4)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, agg in res:
        assert t == 5.0
        assert agg == 5.0 / 8
