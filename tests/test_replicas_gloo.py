"""The multi-rank path (independent replicas, one reduction of the rates) on
CPU with the gloo backend, world size 2."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from md_gpu_gb300.replicas import aggregate_rate, replica_seed  # noqa: E402


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


def test_single_rank_is_local():
    rate, t = aggregate_rate(1000.0, 2.0, 1)
    assert rate == 500000.0 and t == 2.0
