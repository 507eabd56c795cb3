"""The FP64 mode of the force kernels (md_set_precision(ctx, 64)) against the
oracle's FP64 plain form, through the C ABI.

Tolerances (stated):
* FP64 forces vs the oracle's FP64 plain form on the same positions and list:
  RMS relative <= 1e-9 (both FP64; the library rounds each of an atom's 8
  lane sums to 2^-32 kJ/mol/A fixed point, up to 1e-9 kJ/mol/A per atom,
  which is ~1e-9 relative for argon's forces of ~1 kJ/mol/A);
* per-atom energies and sum ff r^2: RMS relative <= 2e-7 (stored as FP32);
* FP32 mode vs FP64 mode on the GPU: RMS relative <= 1e-5 (the path's gate);
* short FP64 runs vs the oracle's FP64 plain-form run: positions within
  1e-8 A and KE within 1e-9 relative after 40 steps; PE within 1e-8 relative
  (per-atom energies are stored in FP32 before their exact fixed-point sum,
  ~4e-6 kJ/mol on the 500-atom total).
"""
import os
import tempfile

import numpy as np
import pytest

import oracle
import golden_util as gu
from md_gpu_gb300 import MD_VV, TERM_ALL, TERM_ANGLE, TERM_BOND, TERM_PAIR
from md_gpu_gb300 import MDSystem
from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import synth

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-9


@pytest.fixture(scope="module", autouse=True)
def _lib():
    mdbuild.build()


@pytest.fixture(scope="module", params=gu.names())
def gcase(request):
    g = gu.load_golden(request.param)
    return request.param, gu.case_from_golden(g)


def _bonded64(case):
    pos4 = case.pos4()
    f = np.zeros((case.natom, 4))
    ep = np.zeros(case.natom)
    arr = lambda k: np.ctypeslib.as_array(getattr(case.fld, k)).astype(np.float32)
    if len(case.bonds):
        oracle.bonds_f64(pos4, case.box, case.bonds, arr("bnd1"), arr("bnd2"), f, ep)
    if len(case.angles):
        oracle.angles_f64(pos4, case.box, case.angles, arr("ang1"), arr("ang2"), f, ep)
    return f, ep


def test_fp64_pair_forces_match_plain_form(gcase):
    name, case = gcase
    orc = gu.oracle_state(case)
    with gu.system_from_case(case) as sim:
        sim.set_precision(64)
        sim.compute_forces(TERM_PAIR, energy=True)
        F = sim.forces()
        ep = sim.energies()
        th = sim.thermo()
    assert gu.rms_rel(F[:, :3], orc["f64"][:, :3]) <= FP64_TOL
    assert gu.rms_rel(F[:, 3], orc["f64"][:, 3]) <= 2e-7
    assert gu.rms_rel(ep, orc["ep64"]) <= 2e-7
    assert abs(th["pe"] - orc["ep64"].sum()) <= 1e-7 * np.abs(orc["ep64"]).sum()


def test_fp64_bonded_forces_match_plain_form(gcase):
    name, case = gcase
    if not len(case.bonds) and not len(case.angles):
        pytest.skip("no bonded terms")
    f, ep = _bonded64(case)
    with gu.system_from_case(case) as sim:
        sim.set_precision(64)
        sim.compute_forces(TERM_BOND | TERM_ANGLE, energy=True)
        F = sim.forces()
        E = sim.energies()
    assert gu.rms_rel(F[:, :3], f[:, :3]) <= FP64_TOL
    assert gu.rms_rel(E, ep) <= 2e-7


def test_fp32_mode_within_gate_of_fp64_mode(gcase):
    """The FP32 kernels against the FP64 mode of the same library, same state."""
    name, case = gcase
    with gu.system_from_case(case) as sim:
        sim.compute_forces(TERM_ALL)
        F32 = sim.forces()
        sim.set_precision(64)
        sim.compute_forces(TERM_ALL)
        F64 = sim.forces()
        sim.set_precision(32)
        sim.compute_forces(TERM_ALL)
        assert np.array_equal(sim.forces(), F32)
    assert gu.rms_rel(F32[:, :3], F64[:, :3]) <= 1e-5


def _write(system):
    td = tempfile.mkdtemp()
    return synth.write_case(system, td, "c")


def test_fp64_velocity_verlet_matches_plain_run():
    case = oracle.load(_write(synth.argon_fcc(ncell=5, seed=4, integrator="vv")))
    x = case.pos.astype(np.float64).copy()
    v = case.vel.astype(np.float64).copy()
    st, rec = oracle.md_plain_run(case, x, v, 40, 1)
    with gu.system_from_case(case, integrator=MD_VV) as sim:
        sim.set_precision(64)
        sim.step(40, energy_every=1)
        hist = sim.history(40)
        pos = sim.positions()
    ke = np.array([h["ke"] for h in hist])
    pe = np.array([h["pe"] for h in hist])
    assert np.abs(ke - rec[:, 0]).max() <= 1e-9 * np.abs(rec[:, 0]).max()
    assert np.abs(pe - rec[:, 1]).max() <= 1e-8 * np.abs(rec[:, 1]).max()
    d = pos - x
    d -= case.box.astype(np.float64) * np.rint(d / case.box.astype(np.float64))
    assert np.abs(d).max() <= 1e-8


def test_fp64_batch_replicas_like_single():
    with tempfile.TemporaryDirectory() as td:
        cases = [oracle.load(synth.write_case(synth.nacl_replica(n, seed=s), os.path.join(td, str(s)), "r"))
                 for n, s in ((600, 1), (900, 2), (1302, 3))]
    kws = [gu.case_arrays(c, integrator=MD_VV) for c in cases]
    with MDSystem.from_batch(kws) as b:
        b.set_precision(64)
        b.compute_forces(TERM_ALL, energy=True)
        Fb = b.forces()
        Eb = b.energies()
        sl = b.replica_slices()
    for kw, s in zip(kws, sl):
        with MDSystem.from_arrays(**kw) as one:
            one.set_precision(64)
            one.compute_forces(TERM_ALL, energy=True)
            assert np.array_equal(one.forces()[:, :3], Fb[s, :3])
            assert np.array_equal(one.energies(), Eb[s])
