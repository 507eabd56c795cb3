"""The reference's step loop (runGPU.cu:44-115) driven through the
reference-compatible entry points (tests/compat/compat_driver.cpp) advances
bit for bit like md_step on the same system: the same kernels run in the
same order (list check and rebuild, forces, energies every timprn steps,
leapfrog; or in the velocity-Verlet form of the loop, integrate_pre before
and integrate_cor after), with the charges the reference's kernels see
(packed into pos.w and decoded in FP32).  config_finish leaves the charges
unpacked in pos.w."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import compat_util as cu
from md_gpu_gb300 import MDSystem, synth
from md_gpu_gb300 import build as mdbuild

pytestmark = pytest.mark.gpu

NSTEPS, TIMPRN = 40, 10


@pytest.fixture(scope="module")
def driver():
    with tempfile.TemporaryDirectory() as td:
        yield cu.build_driver(mdbuild.build(), td)


@pytest.mark.parametrize("enstype,vv", [(0, False), (1, False), (0, True), (1, True)])
def test_reference_loop_matches_md_step(driver, enstype, vv):
    a = synth.to_arrays(synth.nacl_rocksalt(ncell=5, seed=52, nmaxlist=512))
    a["integrator"] = 0
    a["enstype"] = enstype
    n = len(a["itype"])
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        cu.write_input(fin, a, NSTEPS, TIMPRN)
        subprocess.run([driver, fin, fout] + (["vv"] if vv else []), check=True, capture_output=True, timeout=300)
        pos, vel, temper, qback = cu.read_output(fout, n, NSTEPS)
    # velocity Verlet: NVE, or Nose-Hoover for NVT (what integrate_pre selects)
    b = dict(a, charge=cu.packed_charges(a["itype"], a["charge"]), tau_t=100.0,
             integrator=(2 if enstype else 1) if vv else 0)
    with MDSystem.from_arrays(**b) as sim:
        sim.step(NSTEPS, energy_every=TIMPRN)
        assert sim.info()["builds"] >= 2
        X, V = sim.positions(), sim.velocities()
        hist = sim.history(NSTEPS)
    assert np.array_equal(pos, X.astype(np.float32))
    assert np.array_equal(vel, V.astype(np.float32))
    assert np.array_equal(temper, np.array([h["temper"] for h in hist], np.float32))
    t = np.asarray(a["itype"]).astype(np.float32)
    w = t + np.float32(0.1) * (np.asarray(a["charge"], np.float32) + np.float32(5.0))
    assert np.array_equal(qback, (w - t) * np.float32(10.0) - np.float32(5.0))
