"""bench.py's multi-GPU paths on CPU, with gloo ranks.

A single blob does not shard (replicas only): each rank steps its own
replica with its own RNG stream and the job's time is the slowest rank's.
An ensemble of independent blobs shards: ffea_gb300.partition packs the
blobs over the ranks by estimated bytes per step, each rank steps its share
with no exchange, and the results are gathered on the host at the end.

  test_two_replicas_over_gloo    replica seeds, the max-over-ranks time and
                                 the whole-job throughput, world size 2
  test_ensemble_shards_over_gloo two ranks each step their packed share of a
                                 six-blob ensemble with the oracle (FFEA's
                                 step restated, one thread); the gathered
                                 positions, velocities and RNG states equal a
                                 one-process run of all six blobs bit for bit
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ENSEMBLE_RADII = (3.0, 4.5, 2.5, 3.5, 4.0, 3.0)
ENSEMBLE_STEPS = 3


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _init(rank, world, port):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    return dist


def _worker(rank, world, port, out):
    dist = _init(rank, world, port)
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


def _ensemble_blob(i):
    """Blob i of the test ensemble: its mesh, moduli and RNG seed depend on i only."""
    from tests.helpers import spec
    return spec(radius_nm=ENSEMBLE_RADII[i], seed=i, rng_seed=500 + i, shear_mod=3.7e8 * (0.75 + 0.1 * i))


def _step_blobs(indices):
    """{index: (pos, vel, rng state)} after ENSEMBLE_STEPS oracle steps of each blob."""
    from oracle import oracle as O
    res = {}
    for i in indices:
        b = O.blob_from_spec(_ensemble_blob(i))
        assert b.step(ENSEMBLE_STEPS) == 0
        pos, vel, _ = b.nodes()
        res[i] = (pos, vel, b.rng_state())
    return res


def _plan(world):
    from ffea_gb300 import partition as Pt
    costs = [Pt.blob_cost(*Pt.estimate_sizes(r)) for r in ENSEMBLE_RADII]
    return Pt.pack(costs, world)


def _ensemble_worker(rank, world, port, out):
    dist = _init(rank, world, port)
    bins, _ = _plan(world)
    mine = _step_blobs(bins[rank])
    # the only exchange: a host-side gather of the results at the end
    gathered = [None] * world
    dist.all_gather_object(gathered, {i: tuple(np.asarray(a).tobytes() for a in v) for i, v in mine.items()})
    if rank == 0:
        merged = {}
        for g in gathered:
            merged.update(g)
        out["merged"] = merged
        out["bins"] = bins
    dist.destroy_process_group()


def test_ensemble_shards_over_gloo():
    from ffea_gb300 import partition as Pt
    world = 2
    bins, loads = _plan(world)
    assert sorted(i for b in bins for i in b) == list(range(len(ENSEMBLE_RADII)))
    assert all(b for b in bins), "every rank gets blobs"
    assert max(loads) <= 1.35 * min(loads), loads
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_ensemble_worker, args=(world, port, out), nprocs=world, join=True)
        merged = dict(out["merged"])
    single = _step_blobs(range(len(ENSEMBLE_RADII)))
    assert sorted(merged) == sorted(single)
    for i, (pos, vel, st) in single.items():
        assert merged[i] == (pos.tobytes(), vel.tobytes(), st.tobytes()), f"blob {i} differs when sharded"
    # the packer is deterministic and balances a replicated ensemble evenly
    plan, loads4 = Pt.ensemble_plan(ENSEMBLE_RADII, 4)
    assert sorted(x for b in plan for x in b) == [(r, i) for r in range(4) for i in range(len(ENSEMBLE_RADII))]
    assert max(loads4) == pytest.approx(min(loads4))
    assert Pt.ensemble_plan(ENSEMBLE_RADII, 4)[0] == plan
