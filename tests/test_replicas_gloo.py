"""The multi-rank path (independent replicas, one reduction of the rates) on
CPU with the gloo backend, world size 2."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import numpy as np  # noqa: E402

from md_gpu_gb300.replicas import aggregate_rate, gather_per_replica, partition, replica_seed  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    atom_steps = 64000 * 100 * (rank + 1)
    ms = 10.0 + 5.0 * rank
    rate, tmax = aggregate_rate(atom_steps, ms, world)
    out[rank] = (rate, tmax, replica_seed(1, rank))
    dist.destroy_process_group()


def test_two_rank_aggregation():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    total = 64000 * 100 * (1 + 2)
    for r in range(world):
        rate, tmax, seed = out[r]
        assert tmax == 15.0
        assert abs(rate - total / 15e-3) < 1e-6 * rate
    assert out[0][2] != out[1][2]


SIZES = np.random.default_rng(3).integers(256, 8193, 512)


def _partition_worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    idx = partition(SIZES, world, rank)
    # a per-replica observable (two columns) computed by the owner only
    local = np.stack([idx * 1.5, SIZES[idx].astype(np.float64)], 1)
    full = gather_per_replica(local, idx, len(SIZES), world)
    out[rank] = (idx.tolist(), full.tolist())
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_batch_partition_and_gather(world):
    """The replicas of one batch shared out across ranks: every replica on
    exactly one rank, contiguous and balanced by atoms; the per-replica
    results gathered back in replica order on every rank."""
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_partition_worker, args=(world, port, out), nprocs=world, join=True)
    owned = [np.array(out[r][0]) for r in range(world)]
    allidx = np.concatenate(owned)
    assert np.array_equal(np.sort(allidx), np.arange(len(SIZES)))
    assert all(np.all(np.diff(o) == 1) for o in owned if len(o))
    atoms = np.array([SIZES[o].sum() for o in owned])
    assert atoms.max() - SIZES.sum() / world <= SIZES.max()
    expect = np.stack([np.arange(len(SIZES)) * 1.5, SIZES.astype(np.float64)], 1)
    for r in range(world):
        assert np.array_equal(np.array(out[r][1]), expect)
    # one rank: the whole batch, in order
    assert np.array_equal(partition(SIZES, 1, 0), np.arange(len(SIZES)))


def test_single_rank_is_local():
    rate, t = aggregate_rate(1000.0, 2.0, 1)
    assert rate == 500000.0 and t == 2.0
