"""bench.py's multi-GPU path on CPU: two gloo ranks, one replica blob each.

The blob update does not shard a single blob (replicas only): each rank steps
its own replica with its own RNG stream, there is no exchange during stepping,
and the job's time is the slowest rank's.  This checks the replica seeds, the
max-over-ranks reduction and the whole-job throughput with world_size 2.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import oracle as O
    seed = bench.replica_seed(rank)
    st = O.ffea_seed(seed)
    # a rank's "step time": ranks differ on purpose
    t = 1.0 + rank
    t_max = bench.max_over_ranks(t, world, device="cpu")
    out[rank] = (seed, [int(x) for x in st], t_max, bench.aggregate_throughput(1000, 10, world, t_max))
    dist.destroy_process_group()


def test_two_replicas_over_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] != res[1][0]
    assert res[0][1] != res[1][1]  # distinct streams
    assert res[0][2] == res[1][2] == 2.0  # the slowest rank
    assert res[0][3] == pytest.approx(1000 * 10 * 2 / 2.0)
