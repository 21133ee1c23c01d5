"""The multi-GPU path of bench.py is replicas only: each rank runs the whole workload and the job's throughput is
all ranks' units over the slowest rank's time.  Checked here with world_size 2 on the gloo backend (CPU)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        t_local = [2.0, 3.5][rank]
        t_max, value = bench.replica_throughput(t_local, 1000, 4, world, torch.device("cpu"))
        q.put((rank, t_max, value))
    finally:
        dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t_max, value in res:
        assert t_max == 3.5
        assert value == pytest.approx(2 * 1000 * 4 / 3.5)


def test_single_rank_needs_no_process_group():
    import bench
    t_max, value = bench.replica_throughput(2.0, 1000, 4, 1, None)
    assert t_max == 2.0 and value == pytest.approx(2000.0)
