"""Batches of uneven replicas (md_create_batch) against the oracle and
against the same replicas run one at a time.

Tolerances, per replica, as for single systems:
* neighbour lists bit-exact (integer work);
* pair forces RMS relative <= 1e-5 against the FP64 plain form;
* potential energy totals relative <= 1e-6, per-atom energies RMS <= 2e-5;
* a replica in a batch advances bit-for-bit like the same replica alone
  with the same tuning (velocity Verlet NVE: no batch-wide quantity feeds
  back into the trajectory); its kinetic energy agrees to 1e-9 (both sum
  every (atom, axis) term in 2^-32 kJ/mol fixed point, exactly);
* against the FP64 plain-form integrator after 20 steps: KE and PE within
  1e-4 relative, positions within 1e-3 A.
"""
import os
import tempfile

import numpy as np
import pytest

import oracle
import golden_util as gu
from md_gpu_gb300 import MD_LEAPFROG, MD_VV, TERM_PAIR, MDSystem
from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import synth

pytestmark = pytest.mark.gpu

# 216 ions: the cutoff is clamped to the box; 1302 ions sit on a compressed,
# partly vacant lattice (the others fill theirs)
SIZES = [216, 512, 1302, 1728, 2744]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    mdbuild.build()


def _systems(integrator="vv", ensemble="nve", seed=11):
    rng = np.random.default_rng(seed)
    out = []
    for k, n in enumerate(SIZES):
        out.append(synth.nacl_replica(
            n, seed=seed * 100 + k, eps_scale=tuple(rng.uniform(0.9, 1.1, 2)),
            sig_scale=tuple(rng.uniform(0.9, 1.1, 2)), charge_scale=float(rng.uniform(0.9, 1.1)),
            integrator=integrator, ensemble=ensemble, nmaxlist=448))
    return out


@pytest.fixture(scope="module")
def cases():
    with tempfile.TemporaryDirectory() as td:
        return [oracle.load(synth.write_case(s, os.path.join(td, str(k)), "r"))
                for k, s in enumerate(_systems())]


def _batch(cases, **kw):
    return MDSystem.from_batch([gu.case_arrays(c, **kw) for c in cases])


def test_batch_lists_bit_exact(cases):
    with _batch(cases) as b:
        width = 448
        nn, nm = b.neighbor_list(width)
        rows = gu.rows_canonical(nn, nm, b.natom, width)
        for c, sl in zip(cases, b.replica_slices()):
            orc = gu.oracle_state(c)
            assert np.array_equal(nm[sl].astype(np.int64), orc["nm"][:c.natom].astype(np.int64))
            mine = rows[sl].astype(np.int64)
            valid = mine != 0xFFFFFFFF
            mine[valid] -= sl.start
            ref = gu.rows_canonical(orc["nn"], orc["nm"], c.natom, width).astype(np.int64)
            assert np.array_equal(mine, ref)


def test_batch_forces_and_energies_vs_fp64(cases):
    with _batch(cases) as b:
        b.compute_forces(TERM_PAIR, energy=True)
        F = b.forces()
        E = b.energies()
        th = b.replica_thermo()
        for c, sl, t in zip(cases, b.replica_slices(), th):
            orc = gu.oracle_state(c)
            assert gu.rms_rel(F[sl, :3], orc["f64"][:, :3]) <= 1e-5
            assert gu.rms_rel(F[sl, 3], orc["f64"][:, 3]) <= 1e-5
            assert gu.rms_rel(E[sl], orc["ep64"]) <= 2e-5
            pe = float(np.sum(orc["ep64"]))
            assert abs(t["pe"] - pe) <= 1e-6 * abs(pe)


def test_batch_replica_bitwise_like_single(cases):
    """40 VV steps (list rebuilds included): every replica's positions and
    velocities equal those of the replica run alone.  A replica is rebuilt
    only when one of its own atoms moved >= skin/2, so its atom order and
    list order follow the same schedule as when it runs alone."""
    with _batch(cases) as b:
        b.set_tuning(8, 0)
        b.step(40)
        X, V = b.positions(), b.velocities()
        th = b.replica_thermo()
        total = b.thermo()
        assert b.info()["builds"] >= 2
    # per-replica sums are exact integer sums of terms rounded to 2^-32 kJ/mol
    assert abs(sum(t["ke"] for t in th) - total["ke"]) <= 1e-12 * total["ke"]
    for c, sl, t in zip(cases, b.replica_slices(), th):
        with gu.system_from_case(c) as s:
            s.set_tuning(8, 0)
            s.step(40)
            assert np.array_equal(X[sl], s.positions())
            assert np.array_equal(V[sl], s.velocities())
            one = s.thermo()
            assert t["builds"] == one["builds"]   # each replica rebuilds on its own schedule
            assert abs(t["ke"] - one["ke"]) <= 1e-9 * one["ke"]
            assert abs(t["temper"] - one["temper"]) <= 1e-9 * one["temper"]


def test_batch_vv_vs_plain_fp64(cases):
    """Per-replica KE, PE and positions after 20 VV steps against the FP64
    plain-form integrator (all pairs, no list)."""
    with _batch(cases) as b:
        b.step(19)
        b.step(1, energy_every=1)
        X = b.positions()
        th = b.replica_thermo()
    for c, sl, t in zip(cases[:3], b.replica_slices(), th):
        x = c.pos.astype(np.float64).copy()
        v = c.vel.astype(np.float64).copy()
        st, rec = oracle.md_plain_run(c, x, v, 20, 1)
        assert abs(t["ke"] - rec[-1, 0]) <= 1e-4 * abs(rec[-1, 0])
        assert abs(t["pe"] - rec[-1, 1]) <= 1e-4 * abs(rec[-1, 1])
        d = X[sl] - x
        L = c.box.astype(np.float64)
        d -= L * np.rint(d / L)
        assert np.abs(d).max() <= 1e-3


def test_batch_berendsen_leapfrog_per_replica():
    """Leapfrog with a Berendsen thermostat per replica: each replica's scale
    follows its own temperature; trajectories agree with single runs to
    rounding of the FP64 kinetic-energy sums."""
    with tempfile.TemporaryDirectory() as td:
        cs = [oracle.load(synth.write_case(s, os.path.join(td, str(k)), "r"))
              for k, s in enumerate(_systems("leapfrog", "nvt", seed=4)[:3])]
    with _batch(cs) as b:
        b.set_tuning(8, 0)
        b.step(20)
        X = b.positions()
        th = b.replica_thermo()
    for c, sl, t in zip(cs, b.replica_slices(), th):
        with gu.system_from_case(c) as s:
            s.set_tuning(8, 0)
            s.step(20)
            one = s.thermo()
            assert abs(t["lambda_"] - one["lambda_"]) <= 1e-10
            assert abs(t["temper"] / one["temper"] - 1) <= 1e-9
            assert np.abs(X[sl] - s.positions()).max() <= 1e-8
        assert t["lambda_"] != 1.0


def test_batch_autotune_and_graph_replays(cases):
    """Autotuning a batch keeps the forces; graph replays and eager steps
    give the same trajectory."""
    with _batch(cases) as a, _batch(cases) as b:
        a.compute_forces(TERM_PAIR)
        f0 = a.forces()
        pt, lt = a.autotune()
        assert lt == 0
        a.compute_forces(TERM_PAIR)
        assert gu.rms_rel(a.forces()[:, :3], f0[:, :3]) <= 1e-6
        a.set_tuning(pt, 0)
        b.set_tuning(pt, 0)
        # both start from forces evaluated with the same tuning
        for s in (a, b):
            s.set_positions(b.positions())
            s.set_velocities(b.velocities())
        b.set_graphs(False)
        a.step(64)
        b.step(64)
        assert np.array_equal(a.positions(), b.positions())


@pytest.fixture(scope="module")
def water_cases():
    with tempfile.TemporaryDirectory() as td:
        return [oracle.load(synth.write_case(synth.water_grid(nside=n, seed=30 + k, integrator="vv"),
                                             os.path.join(td, "w%d" % k), "w"))
                for k, n in enumerate((8, 9, 8))]


def _water_arrays(c):
    a = gu.case_arrays(c, integrator=MD_VV)
    a["enstype"] = 0
    return a


def test_batch_bonded_replicas(water_cases):
    """Replicas with bonds and angles (flexible water; the H-H pair excluded
    through a zero-force bond): forces against the FP64 plain form (pair,
    bonds, angles) at the start, then 160 VV steps in the batch equal each
    replica run alone, bit for bit (list rebuilds and the remapping of the
    exclusions and bonded lists included)."""
    with MDSystem.from_batch([_water_arrays(c) for c in water_cases]) as b:
        b.set_tuning(8, 0)
        b.compute_forces()
        F = b.forces()
        for c, sl in zip(water_cases, b.replica_slices()):
            orc = gu.oracle_state(c)
            f = orc["f64"].copy()
            ep = np.zeros(c.natom)
            arr = lambda k: np.ctypeslib.as_array(getattr(c.fld, k)).astype(np.float32)
            oracle.bonds_f64(orc["pos4"], c.box, c.bonds, arr("bnd1"), arr("bnd2"), f, ep)
            oracle.angles_f64(orc["pos4"], c.box, c.angles, arr("ang1"), arr("ang2"), f, ep)
            assert gu.rms_rel(F[sl, :3], f[:, :3]) <= 1e-5
    # a fresh batch: compute_forces above re-evaluated the forces without
    # energies (packed pair loop), the first step's half kick after creation
    # uses those of the energy kernel (one entry at a time), like the single runs
    with MDSystem.from_batch([_water_arrays(c) for c in water_cases]) as b:
        b.set_tuning(8, 0)
        b.step(160)
        X, V = b.positions(), b.velocities()
        th = b.replica_thermo()
    assert sum(t["builds"] for t in th) >= 3
    for c, sl, t in zip(water_cases, b.replica_slices(), th):
        with MDSystem.from_arrays(**_water_arrays(c)) as s:
            s.set_tuning(8, 0)
            s.step(160)
            assert np.array_equal(X[sl], s.positions())
            assert np.array_equal(V[sl], s.velocities())
            assert t["builds"] == s.thermo()["builds"]
