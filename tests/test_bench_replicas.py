"""The multi-GPU path of the benchmark is N independent replicas: each rank
times its own queries and rank 0 reports every rank's queries over the
slowest rank's time.  The host-side aggregation runs here as two gloo ranks
on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_env() == (rank, world, rank)
    local_ms = 100.0 + 50.0 * rank  # rank 1 is the slowest
    slowest = bench.max_over_ranks(local_ms, dist, "cpu")
    value = bench.replica_rate(10_000, 5, world, slowest)
    out.put((rank, slowest, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slowest, value in res:
        assert slowest == 150.0  # the max over ranks, on every rank
        assert value == pytest.approx(2 * 10_000 * 5 / 0.150)


def test_single_process_aggregation():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.replica_rate(1000, 2, 1, 500.0) == pytest.approx(4000.0)
