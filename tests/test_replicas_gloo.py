"""Multi-GPU runs are independent replicas, one per rank, with no data-path
collective: the job's time is the slowest rank's, its throughput all ranks'
units over that time.  The aggregation runs here as two gloo ranks on CPU."""
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

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seconds = 1.0 + rank  # rank 1 is the slow one
    slowest = bench.max_over_ranks(seconds, dist, "cpu")
    value = bench.replica_throughput(4000, 100, world, slowest)
    out.put((rank, slowest, value))
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slowest, value in res:
        assert slowest == 2.0
        assert value == 4000 * 100 * 2 / 2.0
