"""Replica parallelism: independent systems per rank, no data-path exchange.

A single md_gpu system is not split across GPUs (that needs a halo exchange
the reference never had).  Several GPUs either each run their own system
with its own seed, or share out the replicas of one batch (partition): each
rank runs its part as a batch of its own, and the only exchanges are on the
host after the run: the per-replica observables or gradients gathered in
replica order (gather_per_replica) and the throughput reduced as total
atom-steps over the slowest rank's time (aggregate_rate).
"""
from __future__ import annotations


def replica_seed(base_seed: int, rank: int) -> int:
    """Seed of the replica a rank runs (distinct per rank, reproducible)."""
    return int(base_seed) + 1000003 * int(rank)


def partition(sizes, world: int, rank: int):
    """The replicas rank `rank` of `world` runs: a contiguous range of
    replica indices, balanced by atom count (a replica goes to the rank whose
    share of the total holds the middle of its atoms), so every replica is
    run by exactly one rank and no rank has more than its share plus one
    replica."""
    import numpy as np
    s = np.asarray(sizes, np.float64)
    if world <= 1 or len(s) == 0:
        return np.arange(len(s))
    mid = np.cumsum(s) - 0.5 * s
    owner = np.minimum((mid * world / s.sum()).astype(np.int64), world - 1)
    return np.flatnonzero(owner == rank)


def gather_per_replica(local, index, nrep: int, world: int):
    """Per-replica results of every rank in replica order: `local` holds one
    row per replica in `index` (this rank's partition); returns an array of
    nrep rows on every rank (torch.distributed, any backend, when world > 1)."""
    import numpy as np
    local = np.asarray(local)
    if world <= 1:
        out = np.zeros((nrep,) + local.shape[1:], local.dtype)
        out[np.asarray(index)] = local
        return out
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, (np.asarray(index), local))
    out = np.zeros((nrep,) + local.shape[1:], local.dtype)
    for idx, vals in parts:
        out[idx] = vals
    return out


def aggregate_rate(atom_steps: float, elapsed_ms: float, world: int, device=None):
    """Whole-job atom-steps/s: sum of atom-steps over ranks / max time over
    ranks.  Uses torch.distributed when world > 1 (any backend)."""
    if world <= 1:
        return atom_steps / (elapsed_ms * 1e-3), elapsed_ms
    import torch
    import torch.distributed as dist
    a = torch.tensor([float(atom_steps)], dtype=torch.float64, device=device)
    t = torch.tensor([float(elapsed_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(a, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(a.item()) / (float(t.item()) * 1e-3), float(t.item())


def equilibrate_batch(replicas, temp: float = 1200.0,
                      stages=((0.5, 10.0, 400), (2.0, 100.0, 200))):
    """Relax and thermalise a list of MDSystem.from_arrays keyword dicts as
    one batch: Berendsen leapfrog NVT stages (dt fs, tau fs, steps) at `temp`.
    Replicas generated on a compressed lattice start far from equilibrium;
    this melts them before a production run.  Returns copies of the dicts
    with positions and velocities replaced by the final state."""
    import numpy as np

    from .system import MD_LEAPFROG, MDSystem
    cur = [dict(r) for r in replicas]
    for dt, tau, n in stages:
        spec = [dict(r, integrator=MD_LEAPFROG, enstype=1, temper_0=temp, dt=dt, tau_t=tau)
                for r in cur]
        with MDSystem.from_batch(spec) as b:
            b.step(int(n))
            X, V = b.positions(), b.velocities()
            slices = b.replica_slices()
        for r, sl in zip(cur, slices):
            r["pos"] = X[sl].astype(np.float32)
            r["vel"] = V[sl].astype(np.float32)
    return cur
