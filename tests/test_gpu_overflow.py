"""Neighbour-list overflow, at set-up and inside a run of steps.

The reference never checks its list's length (neighborlist.cu:284).  Here:
* a context created with too small a capacity, and an upload of compressed
  positions that lengthens the rows, grow the list before any force is
  computed; the list is then bit-exact against the oracle;
* an overflow at a rebuild inside md_step (forced by a test hook that
  shrinks the list and asks for a rebuild) is reported as
  MD_ERR_LIST_OVERFLOW when re-running is switched off, and otherwise the
  call restores the state it saved at its start, grows the list and runs the
  steps again: the trajectory is bit for bit the one of a context whose list
  was large enough and rebuilt at the same step.
"""
import tempfile

import numpy as np
import pytest

import oracle
import golden_util as gu
from md_gpu_gb300 import MDSystem
from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import synth
from md_gpu_gb300.system import MDError, library

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    mdbuild.build()


def _list_matches_oracle(sim, case, pos):
    n = case.natom
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = pos
    pos4[:, 3] = case.q
    p = case.params
    excl = oracle.exclusions(n, case.bonds)
    nn, nm, mx = oracle.nlist(pos4, case.box, case.boxi, oracle.rskinsq(p.skin, p.rcutsq), excl, 1024)
    gnn, gnm = sim.neighbor_list(1024)
    assert np.array_equal(gnm[:n], nm[:n])
    cols, gcols = nn.reshape(-1, nm.shape[0]), gnn.reshape(-1, gnm.shape[0])
    for k in range(int(mx)):
        m = nm[:n] > k
        assert np.array_equal(cols[k, :n][m], gcols[k, :n][m])
    return int(mx)


def test_setup_and_upload_grow_the_list():
    with tempfile.TemporaryDirectory() as td:
        base = synth.write_case(synth.nacl_rocksalt(ncell=5, seed=4, nmaxlist=64), td, "o")
        case = oracle.load(base)
        with MDSystem.from_files(base) as sim:
            info = sim.info()
            assert info["capacity"] >= info["max_neighbors"] > 64
            mx0 = _list_matches_oracle(sim, case, case.pos.astype(np.float32))
            # compress the configuration about the box centre: longer rows
            x = sim.positions() * 0.85
            cap0 = sim.info()["capacity"]
            sim.set_positions(x)
            info = sim.info()
            mx1 = _list_matches_oracle(sim, case, x.astype(np.float32))
            assert mx1 > cap0 >= mx0 and info["capacity"] >= mx1


def _pair(td, seed=6):
    base = synth.write_case(synth.nacl_rocksalt(ncell=6, seed=seed, nmaxlist=512), td, "o")
    return MDSystem.from_files(base), MDSystem.from_files(base)


def test_overflow_inside_a_run_is_reported_without_retry():
    with tempfile.TemporaryDirectory() as td:
        a, b = _pair(td)
        with a, b:
            a.step(16)
            assert library().md_debug_list_capacity(a._ctx, 64, 0) == 0
            with pytest.raises(MDError) as e:
                a.step(8)
            assert e.value.status == 5


def test_overflow_inside_a_run_regrows_and_reruns():
    with tempfile.TemporaryDirectory() as td:
        a, b = _pair(td)
        with a, b:
            a.step(16)
            b.step(16)
            L = library()
            assert L.md_debug_list_capacity(a._ctx, 64, 1) == 0      # overflows at the next rebuild
            assert L.md_debug_list_capacity(b._ctx, 512, 1) == 0     # the same rebuild, room enough
            a.step(40)
            b.step(40)
            assert a.info()["list_regrows"] == 1 and b.info()["list_regrows"] == 0
            assert a.info()["capacity"] >= a.info()["max_neighbors"]
            assert np.array_equal(a.positions(), b.positions())
            assert np.array_equal(a.velocities(), b.velocities())
            assert a.thermo()["temper"] == b.thermo()["temper"]
