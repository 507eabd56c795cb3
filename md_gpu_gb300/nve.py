"""Energy conservation of velocity-Verlet NVE runs: the total energy of each
replica of a batch sampled along a trajectory, and its drift (the slope of a
straight-line fit of E/N against time) in kT per atom per ns.

The replicas advance together in one batch context (md_create_batch); the
per-replica records come from the device ring (md_get_replica_history), read
once per chunk of at most 4096 steps, so the run never waits on the host
between steps.  precision=64 runs the same trajectories with the FP64 force
kernels (md_set_precision), the plain FP64 form the FP32 kernels are compared
with.
"""
from __future__ import annotations

import numpy as np

from .system import MDSystem

RING = 4096   # steps the device keeps per-replica records for


def energy_series(replicas, nsteps: int, every: int, precision: int = 32):
    """Runs `nsteps` steps of a batch (from_batch keyword dicts) with
    energies every `every` steps.  Returns (steps, E): the step numbers of
    the samples and E[sample, replica], the conserved quantity (KE + PE)
    in kJ/mol; sample 0 is the initial state."""
    every = int(every)
    if every < 1 or every > RING:
        raise ValueError("every must lie in [1, 4096]")
    chunk = max(every, (RING // every) * every)
    steps, rows = [], []
    with MDSystem.from_batch(replicas) as b:
        if precision == 64:
            b.set_precision(64)
        t0 = b.replica_thermo()
        steps.append(0)
        rows.append([t["ke"] + t["pe"] for t in t0])
        done = 0
        while done < nsteps:
            k = min(chunk, nsteps - done)
            b.step(k, energy_every=every)
            hist, st = b.replica_history(k)
            for h, s in zip(hist, st):
                if (s - done) % every == 0:    # the first step of each energy graph
                    steps.append(int(s) + 1)
                    rows.append(h[:, 2].tolist())
            done += k
    return np.asarray(steps), np.asarray(rows)


def drift(steps, E, natom, dt_fs: float, kt: float):
    """Per-replica drift of E/N in kT per atom per ns (least-squares slope)."""
    t_ns = np.asarray(steps, np.float64) * dt_fs * 1e-6
    n = np.asarray(natom, np.float64)
    out = []
    for r in range(E.shape[1]):
        out.append(np.polyfit(t_ns, E[:, r] / n[r], 1)[0] / kt)
    return np.asarray(out)


def summary(d):
    """Mean and standard error over replicas."""
    d = np.asarray(d, np.float64)
    se = float(d.std(ddof=1) / np.sqrt(len(d))) if len(d) > 1 else float("nan")
    return float(d.mean()), se
