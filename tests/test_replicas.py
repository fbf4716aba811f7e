"""The multi-GPU form of the benchmark is N independent replicas (one frame per rank, no data-path
collective): the host logic that turns the ranks' times into the whole job's number -- a barrier and an
all-reduce MAX of the elapsed time, then all ranks' samples over the slowest rank's time -- run as two
gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, queue):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        elapsed = bench.replica_max(dist, 0.5 + 0.25 * rank, "cpu")  # rank 1 is the slower replica
        queue.put((rank, elapsed, bench.replica_value(1000, 4, world, elapsed)))
    finally:
        dist.destroy_process_group()


def test_replica_time_is_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [0.75, 0.75]
    assert all(abs(g[2] - 1000 * 4 * 2 / 0.75) < 1e-6 for g in got)
