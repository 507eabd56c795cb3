"""NPT: the Berendsen barostat on the leapfrog with the Berendsen thermostat
(md_set_barostat), against the oracle's FP64 plain-form NPT run
(orc_md_plain_npt) on a 1000-ion NaCl box.

Tolerances over 100 steps (0.2 ps) from the same state: box edge relative
1e-9 (the scale per step is clamped at 1e-4 while the pressure is far from
its target, here for most steps), pressure within 1e-5 relative plus 0.5 bar
(FP32 pair forces against FP64; the pressure is ~3e4 bar), temperature 1e-6
relative, positions 1e-4 A.  An .inp with "ensemble: npt" gives the same
run through md_create_from_files.  A box that shrinks past its cell grid's
margin gets a new cell grid between step chunks, and the run stays on the
FP64 trajectory with a complete list; a box that shrinks below twice the list
radius is reported as MD_ERR_BOX.
"""
import os
import tempfile

import numpy as np
import pytest

import oracle
import golden_util as gu
from md_gpu_gb300 import MDSystem
from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import synth
from md_gpu_gb300.system import MDError

pytestmark = pytest.mark.gpu

P0, TAU_P, BETA = 1.0, 500.0, 2e-5


@pytest.fixture(scope="module", autouse=True)
def _lib():
    mdbuild.build()


def _npt_case(td, ncell=5, seed=7, skin=1.0, **inp):
    sys_ = synth.nacl_rocksalt(ncell=ncell, seed=seed, ensemble="npt", skin=skin, nmaxlist=640)
    sys_.inp.update(press=P0, tau_p=TAU_P, compressibility=BETA, **inp)
    return synth.write_case(sys_, td, "n")


def _gpu_series(sim, nsteps):
    L, P = [], []
    for _ in range(nsteps):
        sim.step(1)
        b, p = sim.replica_boxes()
        L.append(b[0, 0])
        P.append(p[0])
    return np.array(L), np.array(P)


def test_npt_matches_fp64_plain_form():
    with tempfile.TemporaryDirectory() as td:
        base = _npt_case(td)
        case = oracle.load(base)
        x = case.pos.astype(np.float64).copy()
        v = case.vel.astype(np.float64).copy()
        box, rec = oracle.md_plain_npt(case, x, v, 100, P0, TAU_P, BETA)
        a = gu.case_arrays(case)
        assert a["enstype"] == 2
        with MDSystem.from_arrays(**a) as sim:
            sim.set_barostat(P0, TAU_P, BETA)
            L, P = _gpu_series(sim, 100)
            T = sim.thermo()["temper"]
            pos = sim.positions()
        with MDSystem.from_files(base) as sim2:      # the .inp's npt line and extension lines
            L2, P2 = _gpu_series(sim2, 100)
    assert np.abs(L - rec[:, 0]).max() <= 1e-9 * rec[0, 0]
    assert np.all(np.abs(P - rec[:, 1]) <= 1e-5 * np.abs(rec[:, 1]) + 0.5)
    assert abs(T - rec[-1, 2]) <= 1e-6 * rec[-1, 2]
    d = pos - x
    d -= box * np.rint(d / box)
    assert np.abs(d).max() <= 1e-4
    assert np.array_equal(L, L2) and np.array_equal(P, P2)
    assert L[-1] < L[0]          # the box shrinks towards the target pressure


def _missing_pairs(pos, box, rl, nn, nm):
    """Pairs closer than rl - 1e-4 A (minimum image) absent from the list,
    and listed partners farther than rl + 1e-4 A."""
    n = len(pos)
    pt = nm.shape[0]
    cols = nn.reshape(-1, pt)
    missing = far = 0
    for i in range(n):
        d = pos - pos[i]
        d -= box * np.rint(d / box)
        r = np.sqrt((d * d).sum(1))
        r[i] = np.inf
        row = set(int(j) for j in cols[:nm[i], i])
        row.discard(i)
        want = set(np.nonzero(r < rl - 1e-4)[0].tolist())
        missing += len(want - row)
        far += sum(1 for j in row if r[j] > rl + 1e-4)
    return missing, far


def test_npt_regrid_keeps_the_fp64_trajectory():
    """7^3 x 8 ions in a 44.6 A box with a list radius of 14.4 A (skin
    2.4 A): 6 cells of 7.43 A per axis, 3.2% longer than half the list
    radius (stencil +-2).  A target of 1e5 bar shrinks the box by the
    clamped 1e-4 per step; after ~170 steps the cells are within half the
    margin and md_step lays out 5 cells per axis.  300 steps in one call
    follow the FP64 plain-form run, and the list built on the new grid holds
    every pair within the list radius."""
    with tempfile.TemporaryDirectory() as td:
        base = _npt_case(td, ncell=7, seed=8, skin=2.4)
        case = oracle.load(base)
        x = case.pos.astype(np.float64).copy()
        v = case.vel.astype(np.float64).copy()
        box, rec = oracle.md_plain_npt(case, x, v, 300, 1e5, TAU_P, BETA)
        with MDSystem.from_files(base) as sim:
            sim.set_barostat(1e5, TAU_P, BETA)
            assert sim.info()["ncell"] == [6, 6, 6]
            sim.step(300)
            b, p = sim.replica_boxes()
            info = sim.info()
            pos = sim.positions()
            sim.update_neighbors(force=True)
            nn, nm = sim.neighbor_list(640)
    assert info["cell_regrids"] >= 1 and info["ncell"] == [5, 5, 5]
    assert np.abs(b[0] - box).max() <= 1e-9 * box[0]
    assert abs(p[0] - rec[-1, 1]) <= 1e-4 * abs(rec[-1, 1]) + 0.5
    d = pos - x
    d -= box * np.rint(d / box)
    assert np.abs(d).max() <= 1e-3
    rl = float(np.sqrt(case.params.rcutsq)) + 2.4
    missing, far = _missing_pairs(pos, b[0], rl, nn, nm)
    assert missing == 0 and far == 0


def test_npt_regrid_when_the_box_grows():
    """The same 2744-ion box pulled at -1e5 bar grows by the clamped 1e-4
    per step; once a box edge holds a seventh cell of 1.03 times half the
    list radius with 1% to spare (~1600 steps), md_step lays out 7 cells per
    axis, and the list built on that grid holds every pair within the list
    radius."""
    with tempfile.TemporaryDirectory() as td:
        base = _npt_case(td, ncell=7, seed=8, skin=2.4)
        with MDSystem.from_files(base) as sim:
            sim.set_barostat(-1e5, TAU_P, BETA)
            L0 = sim.replica_boxes()[0][0].copy()
            sim.step(1800)
            b, p = sim.replica_boxes()
            info = sim.info()
            pos = sim.positions()
            sim.update_neighbors(force=True)
            nn, nm = sim.neighbor_list(640)
            case = oracle.load(base)
    assert info["cell_regrids"] >= 1 and info["ncell"] == [7, 7, 7]
    assert np.all(p[0] > -1e5)          # the scale stayed clamped at 1 + 1e-4
    # the first step scales by 1 (no pressure measured before it), the other
    # 1799 by the clamped 1 + 1e-4
    assert np.abs(b[0] - L0 * (1.0 + 1e-4) ** 1799).max() <= 1e-9 * L0[0]
    rl = float(np.sqrt(case.params.rcutsq)) + 2.4
    missing, far = _missing_pairs(pos, b[0], rl, nn, nm)
    assert missing == 0 and far == 0


def test_npt_box_below_twice_the_list_radius_is_reported():
    """1000 ions in a 31.86 A box with a list radius of 15.85 A (skin
    3.85 A): a target of 1e5 bar shrinks the box by 1e-4 per step, and after
    ~50 steps it is shorter than twice the list radius."""
    with tempfile.TemporaryDirectory() as td:
        base = _npt_case(td, ncell=5, seed=9, skin=3.85)
        with MDSystem.from_files(base) as sim:
            sim.set_barostat(1e5, TAU_P, BETA)
            with pytest.raises(MDError) as e:
                sim.step(400)
            assert e.value.status == 8
