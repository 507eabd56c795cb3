"""The library against the reference's own CUDA kernels run on the GPU (the
compat-patched copy of its sources, baseline/reference_cuda.py), through the
reference's host entry points: one neighbour-list build and one force
evaluation on the same inputs.

* neighbour lists: the reference GPU kernel's list (neighborlist_nsquared)
  and the library's are equal entry for entry (integer work, bit-exact);
* forces: RMS relative difference <= 1e-5 between the library's FP32 forces
  and the reference kernel's FP32 forces (its rsqrtf, __fdividef and exp2f
  against the library's own approximations), and each within 1e-5 of the
  FP64 plain form.

Skipped where the patched sources are absent (they are made from the
reference tree and travel with the repository).
"""
import os
import tempfile

import numpy as np
import pytest

import oracle
import golden_util as gu
from baseline import reference_cuda as rc
from md_gpu_gb300 import TERM_ALL, MDSystem
from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = {
    "nacl_wolf": lambda: synth.nacl_rocksalt(ncell=6, seed=3, nmaxlist=512),
    "water_wolf_bonded": lambda: synth.water_grid(nside=8, seed=5, nmaxlist=1024),
    "argon_lj": lambda: synth.argon_fcc(ncell=6, seed=2, integrator="leapfrog"),
}


@pytest.fixture(scope="module")
def binary():
    if not rc.have_sources():
        pytest.skip("patched reference sources not present")
    mdbuild.build()
    return rc.build()


@pytest.mark.parametrize("name", sorted(CASES))
def test_list_and_forces_match_reference_gpu_kernels(binary, name):
    with tempfile.TemporaryDirectory() as td:
        base = synth.write_case(CASES[name](), td, "c")
        rc.check_case(base)
        nmax_ref, f_ref, cols_ref = rc.forces(binary, base)
        case = oracle.load(base)
        n = case.natom
        with MDSystem.from_files(base) as sim:
            nn, nm = sim.neighbor_list(int(nmax_ref.max()) + 1)
            sim.compute_forces(TERM_ALL)
            F = sim.forces()
    assert np.array_equal(nm[:n], nmax_ref)
    cols = nn.reshape(-1, nm.shape[0])
    for k in range(int(nmax_ref.max())):
        m = nmax_ref > k
        assert np.array_equal(cols[k, :n][m], cols_ref[k][m]), k
    assert gu.rms_rel(F[:, :3], f_ref[:, :3].astype(np.float64)) <= 1e-5
    orc = gu.oracle_state(case)
    f64 = orc["f64"][:, :3].copy()
    if len(case.bonds) or len(case.angles):
        ep = np.zeros(n)
        f4 = np.zeros((n, 4))
        arr = lambda k: np.ctypeslib.as_array(getattr(case.fld, k)).astype(np.float32)
        if len(case.bonds):
            oracle.bonds_f64(orc["pos4"], case.box, case.bonds, arr("bnd1"), arr("bnd2"), f4, ep)
        if len(case.angles):
            oracle.angles_f64(orc["pos4"], case.box, case.angles, arr("ang1"), arr("ang2"), f4, ep)
        f64 += f4[:, :3]
    assert gu.rms_rel(f_ref[:, :3].astype(np.float64), f64) <= 1e-5
    assert gu.rms_rel(F[:, :3], f64) <= 1e-5
