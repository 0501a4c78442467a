"""Replicas on N ranks (bench.py --gpus N under torchrun): the job's time is the
slowest rank's and its work the sum over ranks. Exercised here with two gloo
ranks on the CPU (the data path has no collective; only these figures are
reduced)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    ms, cells = bench.reduce_max_sum(dist, torch, 10.0 + rank, 1000 * (rank + 1), "cpu")
    out.put((rank, ms, cells))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_report_slowest_time_and_total_cells():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = [out.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, cells in got:
        assert ms == 11.0 and cells == 3000.0, (rank, ms, cells)
