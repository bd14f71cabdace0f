"""Multi-process host logic on CPU (gloo, world size 2).

The path shards over independent systems with no exchange step, so several
GPUs run replicas; the only cross-rank operations are the barrier around the
timed region and the max-over-ranks of the step time that bench.py uses.
This test runs that aggregation, and each rank's replica seed choice, as two
gloo processes on CPU.
"""
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
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 10.0 + 5.0 * rank  # per-rank step time
    agg = bench.reduce_max_ms(ms, dist)
    seed = bench.replica_seed(0, rank)
    val = bench.aggregate_value(1000, world, agg)
    dist.barrier()
    out[rank] = (agg, seed, val)
    dist.destroy_process_group()


def test_two_rank_aggregation():
    world, port = 2, _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    assert out[0][0] == out[1][0] == 15.0  # max over ranks
    assert out[0][1] != out[1][1]  # independent replicas
    assert out[0][2] == out[1][2] == 1000 * 2 / 15e-3
