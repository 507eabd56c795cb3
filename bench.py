#!/usr/bin/env python
"""Benchmark: MD steps of 64000-ion molten NaCl (LJ + Wolf Coulomb, alpha 0.2/A,
rc 12 A, skin 1 A, Berendsen leapfrog NVT at 1200 K, dt 2 fs) on one GB300.

One bench "step" is one segment of --md-steps MD steps (list check and
rebuilds at their natural rate, forces, integration) run through md_step as
captured CUDA graphs (32 steps per graph).  L2 is flushed (512 MB write)
before every timed segment; inside a segment the ~80 MB working set stays
resident, as in any MD run.

The same line carries, under "batched_replicas", the batch workload: 512
NaCl-like replicas of 256..8192 ions (own eps/sigma per type and charge scale
within +-10%), velocity Verlet NVE at dt 2 fs, advanced together by
md_create_batch (one launch per stage, one graph for the batch); and under
"adjoint", gradients per second of a trajectory loss of 64 x 8000-ion NaCl
over 2000 velocity-Verlet steps (md_adjoint_run, checkpoints every 50 steps);
and under "other_systems", the throughput of the 4000-atom argon (velocity
Verlet NVE) and 98304-atom flexible water (Nose-Hoover velocity Verlet,
bonds and angles) systems.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's algorithm on the host cores: the
oracle's FP32 restatement of md_gpu's step loop (O(N^2) list rebuilt on the
skin/2 criterion, full-list pair forces, leapfrog Berendsen), OpenMP over all
host threads (the reference itself has no CPU implementation).
With N > 1 (torchrun) every rank runs an independent replica of the system
(different seed): no data exchange, weak scaling.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "atom-steps/s at 1 GB300 vs plain FP64 at ≤1e-5 force err; adjoint param-grads/s"
UNIT = "atom-steps/s"
WORKLOAD = ("nacl64k: 64000-ion molten NaCl, rocksalt 20^3x8 at 1.5 g/cm^3 melted (Berendsen leapfrog "
            "from the lattice, 2.2 ps at 3000 K then 5 ps at 1200 K; the stored state "
            "md_gpu_gb300/cases/nacl64k_melt.npz), LJ (Lorentz-Berthelot) + Wolf Coulomb alpha 0.2/A rc 12 A "
            "skin 1 A, Berendsen leapfrog NVT 1200 K tau 100 fs, dt 2 fs")
DT_FS = 2.0
# the L2 treatment of the GPU arm, named in both arms' config (the same
# workload; the reference arm runs on host cores)
L2_NOTE = "GPU arm: L2 flushed (512 MB write) before every timed segment"
FLOPS_PER_PAIR = 60.0     # LJ + Wolf per unique pair inside rc (algorithmic count)
# ncu dram__bytes_read.sum + dram__bytes_write.sum of one pair-kernel launch on
# this workload (the melted start state), cold caches (76.81 + 1.72 MB), from
# an ncu capture of k_pair with the tuning bench.py picks; not measured by
# bench.py itself.
PAIR_TRAFFIC_BYTES = 78.53e6


def rank_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class Clocks:
    """nvidia-smi sampled every 50 ms while the timed region runs (entering
    waits, at most 3 s, for the sampler's first line, so that its start-up
    does not fall into the timed region)."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return self
        t0 = time.time()
        while time.time() - t0 < 3.0 and self.proc.poll() is None and os.path.getsize(self.path) == 0:
            time.sleep(0.02)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.proc or not self.path:
            return None
        rows = []
        with open(self.path) as fh:
            for line in fh:
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


# ---- checks in FP64 (numpy / scipy), independent of the library's kernels ----
AS_A = [float(np.float32(a)) for a in (0.254829592, -0.284496736, 1.421413741, -1.453152027, 1.061405429)]
AS_P = float(np.float32(0.3275911))
QFAC = 1389.35427611722


def pairs_within(pos, box, rc):
    """Unordered pairs (i < j) within rc under periodic boundaries (k-d tree)."""
    from scipy.spatial import cKDTree
    L = np.asarray(box, np.float64)
    w = np.mod(np.asarray(pos, np.float64) + 0.5 * L, L)
    w = np.where(w >= L, w - L, w)
    return cKDTree(w, boxsize=L).query_pairs(rc, output_type="ndarray")


def fp64_pair_forces(pos, box, itype, q, lj1, lj2, rcutsq, alfa, pairs):
    """Pair forces of the FP64 plain form: LJ + Wolf with the A&S 7.1.26 erfc
    (the force law of pair_forces.cu:133-205 in FP64), over unordered pairs."""
    x = np.asarray(pos, np.float64)
    L = np.asarray(box, np.float64)
    i, j = pairs[:, 0], pairs[:, 1]
    d = x[i] - x[j]
    d -= L * np.rint(d / L)
    rsq = (d * d).sum(1)
    keep = rsq <= rcutsq
    i, j, d, rsq = i[keep], j[keep], d[keep], rsq[keep]
    r = np.sqrt(rsq)
    ri2 = 1.0 / rsq

    def erfc_as(t_, e_):
        poly = ((((AS_A[4] * t_ + AS_A[3]) * t_ + AS_A[2]) * t_ + AS_A[1]) * t_ + AS_A[0]) * t_
        return poly * e_

    a = float(alfa)
    spi = 2.0 / np.sqrt(np.pi) * a
    rc = np.sqrt(rcutsq)
    ec = np.exp(-a * a * rcutsq)
    W = erfc_as(1.0 / (1.0 + AS_P * a * rc), ec) / rc + spi * ec
    e = np.exp(-a * a * rsq)
    E = erfc_as(1.0 / (1.0 + AS_P * a * r), e)
    qq = QFAC * np.asarray(q, np.float64)[i] * np.asarray(q, np.float64)[j]
    ti, tj = np.asarray(itype)[i], np.asarray(itype)[j]
    l1 = np.asarray(lj1, np.float64).reshape(len(lj1) if np.ndim(lj1) == 2 else int(np.sqrt(np.size(lj1))), -1)
    l2 = np.asarray(lj2, np.float64).reshape(l1.shape)
    ri6 = ri2 * ri2 * ri2
    ff = qq * (spi * e + E / r - W) * ri2 + l1[ti, tj] * ri6 * ri6 * ri2 - l2[ti, tj] * ri6 * ri2
    n = x.shape[0]
    F = np.zeros((n, 3))
    for k in range(3):
        fk = ff * d[:, k]
        F[:, k] = np.bincount(i, fk, n) - np.bincount(j, fk, n)
    return F, int(len(ff))


def drift_leg(args):
    """Total-energy drift of velocity Verlet NVE on LJ argon, 4000 atoms (fcc
    10^3 x 4, rho* 0.8442, T* 0.72, dt 0.5 fs): a batch of seeded replicas
    run by the FP32 kernels over the long horizon and by the FP64 kernels
    (md_set_precision 64, the plain FP64 form on the GPU) over a shorter one;
    per replica the slope of a straight-line fit of E/N against time, in kT
    per atom per ns; mean and standard error over replicas for each, and
    their difference, gated at 1e-4 kT/atom/ns."""
    from md_gpu_gb300 import nve, synth
    R, every, dt, kt, gate = args.drift_reps, 100, 0.5, 0.72, 1e-4
    reps = [synth.to_arrays(synth.argon_fcc(ncell=10, seed=100 + r, integrator="vv")) for r in range(R)]
    natom = [len(a["itype"]) for a in reps]
    out = {}
    for prec, ps in ((32, args.drift_ps), (64, args.drift_fp64_ps)):
        nsteps = int(round(ps * 1000 / dt / every)) * every
        t0 = time.perf_counter()
        st, E = nve.energy_series(reps, nsteps, every, precision=prec)
        wall = time.perf_counter() - t0
        d = nve.drift(st, E, natom, dt, kt)
        m, se = nve.summary(d)
        out[prec] = {"mean": m, "se": se, "horizon_ps": nsteps * dt / 1000, "replicas": R,
                     "seconds": wall, "per_replica": [float(x) for x in d]}
    diff = out[32]["mean"] - out[64]["mean"]
    se_diff = float(np.hypot(out[32]["se"], out[64]["se"]))
    resolved = se_diff <= gate
    return {
        "workload": (f"LJ argon, {R} replicas of 4000 atoms (fcc 10^3 x 4, rho* 0.8442, sigma = 1 A, "
                     "eps = 1 kJ/mol, m = 1 g/mol), T* 0.72 from seeded Maxwell-Boltzmann velocities, "
                     "rc 2.5 (force truncated, energy shifted), skin 0.3, velocity Verlet NVE dt 0.5 fs; "
                     f"E = KE + PE every {every} steps"),
        "unit": "kT/atom/ns",
        "value": out[32]["mean"], "se": out[32]["se"], "horizon_ps": out[32]["horizon_ps"],
        "fp64": {k: out[64][k] for k in ("mean", "se", "horizon_ps", "replicas", "seconds")},
        "fp32_seconds": out[32]["seconds"],
        "difference": diff, "difference_se": se_diff, "gate": gate,
        "gate_passed": bool(resolved and abs(diff) <= gate),
        "gate_resolved": bool(resolved),
        "note": ("FP32 and FP64 kernels on the same seeded replicas; the model (the reference's LJ force "
                 "truncated at rc) drifts by itself, so the gate is on the difference; "
                 "gate_resolved is false when the difference's standard error exceeds the gate")}


def reference_cuda_leg(args, value, e2e_value):
    """The reference's own CUDA build (its sources compat-patched and compiled
    for sm_103a, baseline/reference_cuda.py) on the same melted 64000-ion
    case: its SimulationRun_CUDA loop timed for --ref-cuda-steps steps less a
    0-step run, and one list build + force evaluation of its kernels compared
    with the library's."""
    from baseline import reference_cuda as rc

    import md_gpu_gb300 as md
    from md_gpu_gb300 import synth
    if not rc.have_sources():
        return {"unavailable": "patched reference sources absent (made from the reference tree by build())"}
    binary = rc.build()
    sys_ = synth.nacl_melt64k() if args.ncell == 20 else synth.nacl_rocksalt(ncell=args.ncell, seed=1)
    tmp = tempfile.mkdtemp(prefix="mdref_")
    base = synth.write_case(sys_, os.path.join(tmp, "f"), "ref")
    maxcount = rc.check_case(base)
    nmax_ref, f_ref, cols_ref = rc.forces(binary, base)
    with md.MDSystem.from_files(base) as s:
        nn, nm = s.neighbor_list(int(nmax_ref.max()) + 1)
        s.compute_forces(md.TERM_PAIR)
        F = s.forces()
    n = len(nmax_ref)
    cols = nn.reshape(-1, nm.shape[0])
    same_list = bool(np.array_equal(nm[:n], nmax_ref) and all(
        np.array_equal(cols[k, :n][nmax_ref > k], cols_ref[k][nmax_ref > k]) for k in range(int(nmax_ref.max()))))
    f_ref64 = f_ref[:, :3].astype(np.float64)
    diff = float(np.sqrt(((F[:, :3] - f_ref64) ** 2).sum() / (f_ref64 ** 2).sum()))
    secs, best = rc.time_steps(binary, sys_, tmp, args.ref_cuda_steps)
    rate = n * args.ref_cuda_steps / secs
    return {"value": rate, "unit": UNIT, "md_steps": args.ref_cuda_steps, "seconds": secs,
            "run_seconds": {str(k): v for k, v in best.items()},
            "speedup": value / rate, "e2e_speedup": e2e_value / rate, "target_speedup": 5.0,
            "list_bit_exact_vs_reference_gpu": same_list, "largest_neighbour_count": maxcount,
            "force_rms_rel_diff_vs_reference_gpu": diff,
            "note": ("the reference's sources (src/: the 8 translation units besides athom.cu) with the CUDA 13 "
                     "compat patch (texture reference -> __constant__ pointer, tex1Dfetch -> index, string "
                     "symbols -> symbols) and its parser's heap overflows repaired, nvcc -O3 sm_103a, its "
                     "SimulationRun_CUDA loop (O(N^2) list, 1 thread per atom, host round trips every step) "
                     "from the same melted state, driven by baseline/ref_driver.cu; wall time of "
                     f"{args.ref_cuda_steps} steps less a 0-step run, best of 2")}


def make_case(seed, ncell, tmp):
    """The benchmark system: at the full size (ncell 20) the melted state
    every arm starts from; other sizes a seeded jittered lattice."""
    from md_gpu_gb300 import synth
    sys_ = synth.nacl_melt64k() if ncell == 20 else synth.nacl_rocksalt(ncell=ncell, seed=seed)
    return synth.write_case(sys_, tmp, "nacl")


def cpu_reference_sample(base, samples, warmup, md_steps):
    """Time the oracle's restatement of the reference loop on the host cores:
    one continuing run (the list built once at the start, then rebuilt on the
    reference's skin/2 criterion only), `warmup` untimed slices of md_steps
    steps, then `samples` timed slices of the same run.  Returns (atom-steps/s,
    seconds, threads, builds in the timed slices)."""
    import oracle
    case = oracle.load(base)
    pos4, vel4 = case.pos4(), case.vel4()
    st = oracle.RefLoopState(case.natom, case.params.nmaxlist)
    temper = None
    for _ in range(max(1, warmup)):
        _, temper = oracle.md_ref_run_cont(case, pos4, vel4, md_steps, st, temper=temper)
    builds = 0
    t0 = time.perf_counter()
    for _ in range(samples):
        b, temper = oracle.md_ref_run_cont(case, pos4, vel4, md_steps, st, temper=temper)
        if b < 0:
            raise RuntimeError("reference loop: neighbour list overflow")
        builds += b
    dt = time.perf_counter() - t0
    return case.natom * md_steps * samples / dt, dt, oracle.lib().orc_num_threads(), builds


def run_reference(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return
    with tempfile.TemporaryDirectory() as tmp:
        base = make_case(1, args.ncell, tmp)
        n = 8 * args.ncell ** 3
        ms = args.ref_md_steps
        value, dt, cores, builds = cpu_reference_sample(base, args.steps, args.warmup, ms)
    sample = (f"{args.steps} consecutive slices of {ms} MD steps of one continuing run from the melted "
              f"state (after {max(1, args.warmup)} untimed slices; the O(N^2) list rebuilt only on the "
              f"reference's skin/2 criterion: {builds} builds in the timed slices), N={n}")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": WORKLOAD, "natom": n, "l2": L2_NOTE},
            "run": {"md_steps_per_step": ms, "list_builds_in_timed_region": builds,
                    "parallelism": "host threads (OpenMP)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def system_leg(name, sys_, integrator_name, dt_fs, args, flush):
    """Atom-steps/s of one more single system through md_step (graphs of 32
    steps, L2 flushed before each timed segment)."""
    import torch

    import md_gpu_gb300 as md
    tmp = tempfile.mkdtemp(prefix="mdbench_")
    from md_gpu_gb300 import synth
    base = synth.write_case(sys_, tmp, name)
    with md.MDSystem.from_files(base) as sim:
        pt, lt = sim.autotune()
        sim.step(args.md_steps)
        b0 = sim.info()["builds"]
        ms = []
        for _ in range(args.other_segments):
            flush.zero_()
            torch.cuda.synchronize()
            sim.step(args.md_steps)
            ms.append(sim.last_step_ms())
        info = sim.info()
        n = sim.natom
    steps = args.md_steps * len(ms)
    sps = steps / (sum(ms) * 1e-3)
    return {"value": n * sps, "unit": UNIT, "natom": n, "integrator": integrator_name,
            "ms_per_md_step": sum(ms) / steps, "ns_per_day": sps * dt_fs * 0.0864,
            "list_builds": info["builds"] - b0, "md_steps": steps, "pair_threads_per_atom": pt,
            "pair_entries_per_lane": info["pair_depth"],
            "list_builder": "warp per cell" if lt == 0 else f"{lt} threads per atom"}


def batch_leg(args, flush, rank=0, world=1):
    """Throughput of the 512-replica batch (atom-steps/s over all replicas).
    Under torchrun the replicas are shared out across the ranks (a contiguous
    part per rank, balanced by atoms), each rank runs its part as one batch,
    and the rate is the total atom-steps over the slowest rank's time."""
    import torch

    from md_gpu_gb300 import MDSystem, synth
    from md_gpu_gb300.replicas import aggregate_rate, equilibrate_batch, gather_per_replica, partition
    reps_all = synth.replica_batch(args.nrep, seed=1)
    idx = partition([r.natom for r in reps_all], world, rank)
    reps = [reps_all[i] for i in idx]
    arrs = equilibrate_batch([synth.to_arrays(r) for r in reps])
    sizes = [r.natom for r in reps]
    with MDSystem.from_batch(arrs) as b:
        pt, _ = b.autotune()
        b.step(args.md_steps)
        builds0 = b.info()["builds"]
        rb0 = [t["builds"] for t in b.replica_thermo()]
        ms = []
        for _ in range(args.batch_segments):
            flush.zero_()
            torch.cuda.synchronize()
            b.step(args.md_steps)
            ms.append(b.last_step_ms())
        info = b.info()
        th = b.replica_thermo()
        pair_ms = b.time_pair(20)
    steps = args.md_steps * len(ms)
    rebuilt = sum(t["builds"] for t in th) - sum(rb0)
    value, tmax = aggregate_rate(sum(sizes) * steps, sum(ms), world, device="cuda")
    temps = gather_per_replica(np.array([t["temper"] for t in th]), idx, len(reps_all), world)
    sizes_all = [r.natom for r in reps_all]
    return {
        "workload": (f"{args.nrep} NaCl-like replicas, N uniform in [256, 8192] (seed 1), 1.5 g/cm^3, "
                     "eps/sigma per type and charge scale uniform within +-10% of the molten-NaCl "
                     "values, Wolf alpha 0.2/A, rc 12 A (clamped to L/2 - skin for the smallest boxes), "
                     "skin 1 A, velocity Verlet NVE dt 2 fs, melted first by Berendsen leapfrog "
                     "(400 steps dt 0.5 fs tau 10 fs, 200 steps dt 2 fs tau 100 fs) at 1200 K"),
        "value": value, "unit": UNIT, "ranks": world, "replicas_per_rank_0": len(sizes),
        "natom": int(sum(sizes_all)), "nrep": len(sizes_all), "min_natom": int(min(sizes_all)),
        "max_natom": int(max(sizes_all)), "md_steps": steps, "ms_per_md_step": tmax / steps,
        "pair_ms": pair_ms, "pair_threads_per_atom": pt, "pair_entries_per_lane": info["pair_depth"],
        "batch_rebuild_events": info["builds"] - builds0,
        "replica_rebuilds_per_replica_step": rebuilt / (len(sizes) * steps),
        "temperature_K": {"min": float(temps.min()), "mean": float(temps.mean()), "max": float(temps.max())},
        "l2": "flushed (512 MB write) before every timed segment",
    }


def adjoint_leg(args, rank=0, world=1):
    """Differentiable MD: gradients of <U>/N + RDF loss of 64 x 8000-ion NaCl
    over 2000 VV steps w.r.t. (eps_Na, sigma_Na, eps_Cl, sigma_Cl, charge
    scale), by the library's adjoint with checkpoints every 50 steps.  Under
    torchrun the replicas are shared out across the ranks and the gradients
    gathered in replica order; the time is the slowest rank's."""
    import torch

    from md_gpu_gb300 import MDSystem, params, synth
    from md_gpu_gb300.replicas import gather_per_replica, partition
    nrep_all, natom, K = args.adj_nrep, args.adj_natom, args.adj_steps
    mine = partition([natom] * nrep_all, world, rank)
    nrep = len(mine)
    eps = np.array([synth.NACL_LJ["Na"][1], synth.NACL_LJ["Cl"][1]]) * synth.KCAL
    sig = np.array([synth.NACL_LJ["Na"][0], synth.NACL_LJ["Cl"][0]])

    def batch(scale):
        l1, l2 = params.lb_tables(eps * scale, sig * scale)
        out = []
        for r in mine:
            a = synth.to_arrays(synth.nacl_replica(natom, seed=7000 + int(r), integrator="vv", ensemble="nve"))
            a.update(lj1=l1.astype(np.float32), lj2=l2.astype(np.float32),
                     charge=(a["charge"] * scale).astype(np.float32))
            out.append(a)
        return out

    kw = dict(checkpoint=50, nbins=200, dr=0.05, sigma=0.05)
    with MDSystem.from_batch(batch(1.05)) as b:
        target = b.adjoint(K, gradient=False, **kw)["gbar"]
    with MDSystem.from_batch(batch(1.0)) as b:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fwd = b.adjoint(K, gradient=False, target=target, **kw)
        t_fwd = time.perf_counter() - t0
    with MDSystem.from_batch(batch(1.0)) as b:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = b.adjoint(K, gradient=True, target=target, **kw)
        t_adj = time.perf_counter() - t0
    grads = []
    for r in range(nrep):
        de, ds = params.lb_chain(out["dlj1"][r], out["dlj2"][r], eps, sig)
        grads.append([de[0], ds[0], de[1], ds[1], out["dlns"][r]])
    grads = gather_per_replica(np.array(grads).reshape(-1, 5), mine, nrep_all, world)
    n_grads = grads.size
    if world > 1:   # the slowest rank's times
        import torch.distributed as dist
        tt = torch.tensor([t_adj, t_fwd], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_adj, t_fwd = float(tt[0]), float(tt[1])
    # the stated baseline: per-system plain FP64 runs on the same GPU, central
    # differences of the five parameters (two K-step runs each) of one replica
    one = batch(1.0)[0]
    with MDSystem.from_arrays(**one) as s64:
        s64.set_precision(64)
        s64.step(64)
        n64 = min(K, 512)
        ms64 = 0.0
        for _ in range(2):
            s64.step(n64)
            ms64 += s64.last_step_ms()
        ms_per_step64 = ms64 / (2 * n64)
    fp64_rate = 5.0 / (10 * K * ms_per_step64 * 1e-3)
    return {
        "workload": (f"{nrep_all} replicas of {natom}-ion molten NaCl (LJ + Wolf, rc 12 A), {K} velocity-Verlet "
                     "NVE steps at dt 2 fs from 1200 K; loss = <U>/N + sum_b (gbar_b - target_b)^2 of the "
                     "Gaussian-smoothed Na-Cl RDF (200 bins of 0.05 A, sigma 0.05 A), target from the same "
                     "run at eps, sigma and charges +5%; gradients w.r.t. eps_Na, sigma_Na, eps_Cl, "
                     "sigma_Cl and the charge scale; checkpoints every 50 steps"),
        "value": n_grads / t_adj, "unit": "param-grads/s", "seconds": t_adj,
        "forward_seconds": t_fwd,
        "central_difference_equivalent": {
            "value": n_grads / (10 * t_fwd), "unit": "param-grads/s",
            "note": "10 forward runs of the same batch (two per parameter), FP32 forward"},
        "fp64_per_system": {
            "value": fp64_rate, "unit": "param-grads/s", "ms_per_md_step": ms_per_step64,
            "note": (f"central differences of the 5 parameters by plain FP64 runs (md_set_precision 64) of "
                     f"one {natom}-ion replica at a time: 10 runs of {K} steps per replica, each step timed "
                     f"over {2 * n64} steps (CUDA events)")},
        "vs_fp64_per_system": (n_grads / t_adj) / fp64_rate, "vs_fp64_per_system_target": 10.0,
        "loss_mean": float(out["loss"].mean()), "loss_forward_only_mean": float(fwd["loss"].mean()),
        "grad_mean": grads.mean(0).tolist(),
    }


def run_ours(args):
    import torch
    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    from md_gpu_gb300 import build as mdbuild
    mdbuild.build()
    import md_gpu_gb300 as md

    from md_gpu_gb300.replicas import aggregate_rate, replica_seed
    tmp = tempfile.mkdtemp(prefix="mdbench_")
    base = make_case(replica_seed(1, rank), args.ncell, tmp)
    sim = md.MDSystem.from_files(base)
    n = sim.natom
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    tuned = sim.autotune() if not args.no_autotune else None
    if tuned is None and args.tuning:
        # fixed settings (profiling: timings under a profiler would mislead the tuner)
        pt, depth, lt, fused, inline = (int(v) for v in args.tuning.split(","))
        sim.set_tuning(pt, lt, depth)
        sim.set_fused_step(fused)
        sim.set_graph_rebuild(inline)
    if args.eager:
        sim.set_graphs(False)

    for _ in range(args.warmup):
        sim.step(args.md_steps)
    builds0 = sim.info()["builds"]

    seg_ms = []
    barrier()
    with Clocks(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            sim.step(args.md_steps)
            seg_ms.append(sim.last_step_ms())
        barrier()
    clocks = clk.summary()
    info = sim.info()
    builds = info["builds"] - builds0
    value, total_ms = aggregate_rate(n * args.md_steps * args.steps, float(sum(seg_ms)), world,
                                     device="cuda")
    md_steps_per_s = args.md_steps * args.steps / (total_ms * 1e-3)

    # legs over batches of replicas: every rank runs its share of the replicas
    extra_batch = batch_leg(args, flush, rank, world) if args.nrep > 0 else None
    extra_adj = adjoint_leg(args, rank, world) if args.adj_nrep > 0 else None
    extra = {}
    if rank == 0:
        # roofline of the dominant kernel (pair forces), timed alone on the same state
        from md_gpu_gb300 import synth
        pair_ms = sim.time_pair(50)
        arrs = synth.to_arrays(synth.nacl_rocksalt(ncell=args.ncell, seed=replica_seed(1, rank)))
        pos = sim.positions().astype(np.float32).astype(np.float64)
        rc = float(np.sqrt(arrs["rcutsq"]))
        pc = len(pairs_within(pos, arrs["box"], rc))
        achieved = FLOPS_PER_PAIR * pc / (pair_ms * 1e-3) / 1e12
        peak = md.fp32_peak_tflops()
        roof = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": PAIR_TRAFFIC_BYTES,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_pair launch "
                                  "on this state (a separate capture, cold caches), not measured by this run",
                "kernel": f"k_pair<Wolf> (LJ + Wolf, full list, {info['pair_tpa']} lanes per atom)",
                "pair_ms": pair_ms, "pairs_inside_rc": int(pc), "flops_per_pair": FLOPS_PER_PAIR,
                "peak_source": "measured FP32 FMA probe (md_probe_fp32_peak); no FP32 entry in "
                               "MEASURED_PEAKS.json"}
        # accuracy of the first frame against the FP64 plain form
        with md.MDSystem.from_files(base) as fresh:
            fresh.compute_forces(md.TERM_PAIR)
            F = fresh.forces()
            x0 = fresh.positions().astype(np.float32).astype(np.float64)
        f64, _ = fp64_pair_forces(x0, arrs["box"], arrs["itype"], arrs["charge"], arrs["lj1"], arrs["lj2"],
                                  float(np.float32(arrs["rcutsq"])), arrs["alfa"],
                                  pairs_within(x0, arrs["box"], rc * 1.001))
        err = float(np.sqrt(((F[:, :3] - f64) ** 2).sum() / (f64 ** 2).sum()))
        # end to end through the C ABI from pinned host buffers
        hp = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
        hv = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
        hp[:] = sim.positions()
        hv[:] = sim.velocities()
        e2e_reps = max(1, min(args.steps, 5))
        t0 = time.perf_counter()
        for _ in range(e2e_reps):
            sim.run_host(hp, hv, args.md_steps, inplace=True, raw_records=True)
        e2e_dt = (time.perf_counter() - t0) / e2e_reps
        e2e = {"value": n * args.md_steps / e2e_dt, "unit": UNIT,
               "h2d_bytes_per_step": 2 * 3 * n * 8,
               "d2h_bytes_per_step": 2 * 3 * n * 8 + args.md_steps * 72,
               "call": "md_run_host (upload pos/vel, list build, md_steps steps, download records + pos/vel)"}
        ref_cuda = reference_cuda_leg(args, value, e2e["value"]) if args.ref_cuda_steps > 0 else None
        others = {}
        if args.other_segments > 0:
            from md_gpu_gb300 import synth
            others["argon4000"] = dict(
                workload=("plain LJ argon, 4000 atoms fcc 10^3 x 4, rho* 0.8442, sigma = 1 A, eps = 1 kJ/mol, "
                          "m = 1 g/mol, rc 2.5, skin 0.3, T* 0.72, velocity Verlet NVE dt 0.5 fs"),
                **system_leg("argon", synth.argon_fcc(10, seed=1, integrator="vv"), "velocity Verlet NVE",
                             0.5, args, flush))
            import dataclasses
            melt = synth.nacl_melt64k() if args.ncell == 20 else synth.nacl_rocksalt(ncell=args.ncell, seed=1)
            npt_inp = dict(melt.inp, ensemble="npt", press=1.0, tau_p=1000.0, compressibility=4.5e-5)
            others["nacl64k_npt"] = dict(
                workload=("the benchmark's melted 64000-ion NaCl at constant pressure: Berendsen leapfrog "
                          "with the Berendsen thermostat (1200 K, tau 100 fs) and barostat (1 bar, tau_p "
                          "1000 fs, compressibility 4.5e-5/bar), dt 2 fs; a batch of one replica (the box "
                          "read by the kernels from device memory)"),
                **system_leg("nacl_npt", dataclasses.replace(melt, inp=npt_inp),
                             "Berendsen leapfrog NPT", 2.0, args, flush))
            pme_inp = dict(melt.inp, cutoff=(12.0, 2), pme_spacing=1.2)
            others["nacl64k_pme"] = dict(
                workload=("the benchmark's melted 64000-ion NaCl with Ewald electrostatics in place of Wolf: "
                          "the real-space erfc term (alpha = 3.09/rc = 0.2575/A, rc 12 A, skin 1 A) plus smooth "
                          "particle-mesh Ewald on a 112^3 grid (spacing at most 1.2 A, cubic B-splines), Berendsen "
                          "leapfrog NVT 1200 K, dt 2 fs"),
                **system_leg("nacl_pme", dataclasses.replace(melt, inp=pme_inp),
                             "Berendsen leapfrog NVT with PME", 2.0, args, flush))
            others["water98k"] = dict(
                workload=("flexible 3-site water, 32768 molecules (98304 atoms) at 0.997 g/cm^3, harmonic "
                          "O-H bonds and H-O-H angles, H-H excluded, Wolf alpha 0.2/A rc 10 A skin 1 A, "
                          "Nose-Hoover velocity Verlet 300 K, dt 0.5 fs"),
                **system_leg("water", synth.water_grid(32, seed=1), "Nose-Hoover velocity Verlet", 0.5,
                             args, flush))
        cpu_v, cpu_dt, cores, cpu_builds = cpu_reference_sample(base, 2, 1, args.ref_md_steps)
        extra = {"roofline": roof, "e2e": e2e, "force_rms_rel_err_vs_fp64": err, "nve_drift": drift_leg(args) if args.drift_reps > 0 else None,
                 "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cores, "kind": "port",
                                  "sample": f"2 consecutive slices of {args.ref_md_steps} MD steps of one "
                                            "continuing run from the melted state (after one untimed slice; "
                                            f"{cpu_builds} O(N^2) builds on the skin/2 criterion), oracle "
                                            "FP32 restatement of the reference's loop, OpenMP"}}
        if ref_cuda is not None:
            extra["reference_cuda"] = ref_cuda
        if args.nrep > 0:
            extra["batched_replicas"] = extra_batch
        if extra_adj is not None:
            extra["adjoint"] = extra_adj
        if others:
            extra["other_systems"] = others
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": ("synthetic (seeded rocksalt lattice with 0.25 A jitter and Maxwell-Boltzmann velocities, "
                     "melted)" if args.ncell == 20 else
                     "synthetic (seeded rocksalt lattice with 0.25 A jitter, Maxwell-Boltzmann velocities)"),
            "config": {"workload": WORKLOAD, "natom": n, "l2": L2_NOTE},
            "run": {"md_steps_per_step": args.md_steps,
                    "parallelism": "replicas" if world > 1 else "single system",
                    "ns_per_day": md_steps_per_s * DT_FS * 0.0864,
                    "list_builds_in_timed_region": builds,
                    "pair_threads_per_atom": info["pair_tpa"],
                    "pair_entries_per_lane": info["pair_depth"],
                    "step_kernels": "pair+leapfrog fused" if info["fused_step"] else "pair, leapfrog",
                    "rebuild_in_graph": "inline passes" if info["rebuild_inline"] else "conditional node",
                    "list_builder": "warp per cell" if info["list_tpa"] == 0
                    else f"{info['list_tpa']} threads per atom",
                    "autotuned": tuned is not None,
                    "launch": "eager (profiling)" if args.eager else "CUDA graphs, 32 steps each"},
            "gpu_launches": (args.steps * (args.md_steps // 32 * info["kernels_per_graph"] +
                                           args.md_steps * info["kernels_per_step"]) +
                             builds * info["kernels_per_rebuild"]),
            "clocks": clocks}
    line.update(extra)
    if rank == 0:
        print(json.dumps(line), flush=True)
    sim.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--md-steps", type=int, default=128, help="MD steps per bench step (multiple of 32)")
    ap.add_argument("--nrep", type=int, default=512, help="replicas of the batch leg (0: skip it)")
    ap.add_argument("--batch-segments", type=int, default=4)
    ap.add_argument("--adj-nrep", type=int, default=64, help="replicas of the adjoint leg (0: skip it)")
    ap.add_argument("--adj-natom", type=int, default=8000)
    ap.add_argument("--adj-steps", type=int, default=2000)
    ap.add_argument("--other-segments", type=int, default=3,
                    help="timed segments of the argon and water systems (0: skip them)")
    ap.add_argument("--ref-md-steps", type=int, default=32,
                    help="MD steps per timed slice of the CPU reference loop (slices of one continuing run)")
    ap.add_argument("--ref-cuda-steps", type=int, default=1000,
                    help="steps of the reference's own CUDA loop timed beside the library (0: skip)")
    ap.add_argument("--drift-reps", type=int, default=16, help="argon replicas of the NVE drift leg (0: skip)")
    ap.add_argument("--drift-ps", type=float, default=100.0, help="FP32 horizon of the drift leg, ps")
    ap.add_argument("--drift-fp64-ps", type=float, default=10.0, help="FP64 horizon of the drift leg, ps")
    ap.add_argument("--ncell", type=int, default=20)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tuning", default="",
                    help="with --no-autotune: pair_tpa,pair_depth,list_tpa,fused,inline (e.g. 8,2,0,1,1)")
    ap.add_argument("--eager", action="store_true",
                    help="launch every step's kernels eagerly instead of replaying graphs (for profilers)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    args.md_steps = max(32, (args.md_steps + 31) // 32 * 32)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
