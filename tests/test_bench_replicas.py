"""The replica path of bench.py (N > 1 ranks): max-over-ranks timing and the
whole-job throughput, exercised with world_size 2 over gloo on the CPU."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    d = bench.init_dist(world, "gloo")
    mine = 1.5 + rank   # rank 1 is the slowest replica
    mx = bench.reduce_max(d, mine)
    out[rank] = (mx, bench.aggregate_throughput(10_000 * 20, world, mx))
    d.barrier()
    d.destroy_process_group()


def test_two_rank_replica_aggregation():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    assert out[0][0] == out[1][0] == 2.5
    assert out[0][1] == pytest.approx(2 * 10_000 * 20 / 2.5)


def test_single_rank_is_identity():
    import bench
    assert bench.reduce_max(None, 3.25) == 3.25
    assert bench.aggregate_throughput(100, 1, 2.0) == 50.0
