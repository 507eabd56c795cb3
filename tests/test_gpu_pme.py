"""Smooth particle-mesh Ewald (md_set_pme, lkspace 2) against the FP64 Ewald
oracle (oracle/ewald.py, itself pinned to the exact Ewald sum on the CPU).

Tolerances: the reciprocal forces within 1e-5 RMS relative of the FP64 SPME
on the same grid (FP32 splines and transforms, a 2^-20 fixed-point charge
grid), the energies within 1e-6 relative; the full Coulomb force (real +
reciprocal) within 3e-4 RMS relative of the exact Ewald sum at a 0.5 A grid
(the SPME discretisation error); steps in graphs and eager launches agree
bit for bit, and velocity-Verlet NVE keeps the total energy within 1e-4.
"""
import math
import tempfile

import numpy as np
import pytest

import oracle
from oracle import ewald as ew
from md_gpu_gb300 import MDSystem, TERM_PAIR, TERM_RECIP
from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import synth
from md_gpu_gb300.system import MDError

pytestmark = pytest.mark.gpu

NO_LJ = [(1, 1, "LJ", 1.0, 0.0), (1, 2, "LJ", 1.0, 0.0), (2, 2, "LJ", 1.0, 0.0)]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    mdbuild.build()


def _rms_rel(f, g):
    return float(np.sqrt(((f - g) ** 2).sum() / (g ** 2).sum()))


def _nacl(td, ncell=5, rc=10.0, lj=True, name="p", pme_spacing=None, **kw):
    s = synth.nacl_rocksalt(ncell=ncell, seed=11, rc=rc, nmaxlist=512, vdw=None if lj else NO_LJ, **kw)
    s.inp["cutoff"] = (rc, 2)
    if pme_spacing is not None:
        s.inp["pme_spacing"] = pme_spacing
    return synth.write_case(s, td, name)


def _inputs(case):
    return (float(case.params.alfa), case.q.astype(np.float64), case.box.astype(np.float64))


@pytest.mark.parametrize("grid", [(32, 32, 32), (24, 32, 40)])
def test_recip_matches_fp64_spme(grid):
    """On a cubic grid and on one with a different size per axis (the
    axes' roles in the bricks, transforms and tables)."""
    with tempfile.TemporaryDirectory() as td:
        base = _nacl(td)
        case = oracle.load(base)
        with MDSystem.from_files(base) as sim:
            sim.set_pme(*grid)
            assert sim.info()["pme_grid"] == list(grid)
            sim.compute_forces(TERM_RECIP, energy=True)
            F = sim.forces()[:, :3]
            E = sim.energies()
            x = sim.positions()
            sim.compute_forces(TERM_RECIP, energy=True)
            F2 = sim.forces()[:, :3]
    alpha, q, box = _inputs(case)
    e, f, e_atom = ew.spme_recip(x, q, box, grid, alpha)
    e_atom = e_atom - ew.QFAC * alpha / math.sqrt(math.pi) * q * q
    assert np.array_equal(F, F2)                       # the same grid, bit for bit
    assert _rms_rel(F, f) <= 1e-5
    assert abs(E.sum() - e_atom.sum()) <= 1e-6 * abs(e_atom.sum())
    assert np.abs(E - e_atom).max() <= 1e-4 * np.abs(e_atom).max()


def test_ewald_sum_matches_the_exact_sum():
    """Point charges (no LJ) on the 1000-ion rocksalt: real-space pair term
    plus PME on a 64^3 grid (0.5 A) against the exact Ewald sum."""
    with tempfile.TemporaryDirectory() as td:
        base = _nacl(td, lj=False)
        case = oracle.load(base)
        with MDSystem.from_files(base) as sim:
            sim.set_pme(64)
            sim.compute_forces(TERM_PAIR | TERM_RECIP, energy=True)
            F = sim.forces()[:, :3]
            E = sim.energies()
            x = sim.positions()
    alpha, q, box = _inputs(case)
    rc = float(np.sqrt(np.float32(case.params.rcutsq)))
    er, fr = ew.ewald_real(x, q, box, alpha, rc)
    ek, fk = ew.ewald_recip_exact(x, q, box, alpha, 12)
    et = er + ek + ew.self_energy(q, alpha)
    assert _rms_rel(F, fr + fk) <= 3e-4
    assert abs(E.sum() - et) <= 1e-4 * abs(et)


def test_recip_with_exclusions_matches_fp64():
    """Flexible water (O-H and H-H excluded): the reciprocal sum less each
    atom's excluded partners' erf term."""
    s = synth.water_grid(nside=8, seed=5, integrator="vv")
    s.inp["cutoff"] = (10.0, 2)
    with tempfile.TemporaryDirectory() as td:
        base = synth.write_case(s, td, "w")
        case = oracle.load(base)
        with MDSystem.from_files(base) as sim:
            sim.set_pme(32)
            sim.compute_forces(TERM_RECIP, energy=True)
            F = sim.forces()[:, :3]
            E = sim.energies()
            x = sim.positions()
    alpha, q, box = _inputs(case)
    n = len(q)
    ex = oracle.exclusions(n, case.bonds)
    excl = [[int(j) for j in row if j < n] for row in ex]
    e, f, e_atom = ew.spme_recip(x, q, box, (32, 32, 32), alpha)
    ec, fc = ew.excluded_correction(x, q, box, alpha, excl)
    et = e + ec + ew.self_energy(q, alpha)
    assert _rms_rel(F, f + fc) <= 1e-5
    assert abs(E.sum() - et) <= 1e-5 * abs(et)


def test_pme_steps_graphs_eager_and_energy():
    """Velocity Verlet NVE with PME (1 fs): step graphs and eager launches
    advance bit for bit alike, and the total energy of the energy steps of
    400 steps stays within 2e-4 of the first (the same run without the
    reciprocal sum, i.e. a truncated Coulomb force, is not held to it)."""
    with tempfile.TemporaryDirectory() as td:
        base = _nacl(td, ensemble="nve", integrator="vv", dt=1.0)
        out = []
        for graphs in (True, False):
            with MDSystem.from_files(base) as sim:
                sim.set_pme(32)
                sim.set_graphs(graphs)
                sim.step(400, energy_every=20)
                hist = [h for h in sim.history(400) if h["flags"] & 1]
                out.append((sim.positions(), np.array([h["ke"] + h["pe"] for h in hist]), sim.info()))
    (x0, e, info), (x1, e1, _) = out
    assert np.array_equal(x0, x1) and np.array_equal(e, e1)
    assert len(e) == 20
    assert info["builds"] >= 2 and not info["fused_step"]
    assert np.abs(e - e[0]).max() <= 2e-4 * abs(e[0])


def test_pme_arguments_and_unsupported_cases():
    with tempfile.TemporaryDirectory() as td:
        base = _nacl(td, name="a", pme_spacing=1.0)
        with MDSystem.from_files(base) as sim:      # the .inp's pme_spacing line
            assert sim.info()["pme_grid"] == [32, 32, 32]
            with pytest.raises(MDError) as e:
                sim.set_pme(20)                     # not a multiple of 8
            assert e.value.status == 1
            with pytest.raises(MDError) as e:
                sim.set_type_exclusions(np.zeros(8, np.uint32))
            assert e.value.status == 7
            sim.set_pme(0)
            assert sim.info()["pme_grid"] == [0, 0, 0]
        s = synth.nacl_rocksalt(ncell=5, seed=11, rc=10.0, nmaxlist=512)   # Wolf (lkspace 1)
        with MDSystem.from_files(synth.write_case(s, td, "b")) as sim:
            with pytest.raises(MDError) as e:
                sim.set_pme(32)
            assert e.value.status == 7
