"""bench.py's multi-process aggregation on CPU (gloo, world size 2): each
replica reports its own time, the job takes the slowest, and the whole-job
rate counts every replica's sweeps."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ms = 10.0 * (rank + 1)                       # replica times 10 ms and 20 ms
    got = bench.max_over_ranks(ms, "cpu")
    out[rank] = (got, bench.whole_job_rate(40, world, got))
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    for rank in (0, 1):
        ms, rate = out[rank]
        assert ms == 20.0
        assert rate == pytest.approx(2 * 40 / 0.020)
