"""Replica parallelism: one independent system per rank, no data exchange.

A single md_gpu system is not split across GPUs (that needs a halo exchange
the reference never had); several GPUs each run their own replica with its
own seed.  The only collective is the end-of-run reduction of the throughput
numbers: total atom-steps summed over ranks, time taken as the slowest rank.
"""
from __future__ import annotations


def replica_seed(base_seed: int, rank: int) -> int:
    """Seed of the replica a rank runs (distinct per rank, reproducible)."""
    return int(base_seed) + 1000003 * int(rank)


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
