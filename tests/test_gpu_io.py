"""Trajectory (XYZ) and restart files.

* md_write_xyz writes full-precision frames in original atom order with the
  .fld's element names; appended frames form a trajectory.
* md_write_restart / md_read_restart carry a single system's exact state
  (positions, velocities, step count, thermostat state; Berendsen leapfrog
  and Nose-Hoover velocity Verlet with bonded terms).
"""
import os
import tempfile

import numpy as np
import pytest

from md_gpu_gb300 import MDSystem, synth
from md_gpu_gb300 import build as mdbuild

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    mdbuild.build()


def _read_xyz(path):
    frames = []
    with open(path) as fh:
        lines = fh.read().splitlines()
    k = 0
    while k < len(lines):
        n = int(lines[k])
        comment = lines[k + 1]
        names, xyz = [], []
        for line in lines[k + 2:k + 2 + n]:
            f = line.split()
            names.append(f[0])
            xyz.append([float(v) for v in f[1:4]])
        frames.append((comment, names, np.array(xyz)))
        k += 2 + n
    return frames


def test_xyz_trajectory():
    with tempfile.TemporaryDirectory() as td:
        base = synth.write_case(synth.nacl_rocksalt(ncell=5, seed=61, nmaxlist=512), td, "nacl")
        path = os.path.join(td, "traj.xyz")
        with MDSystem.from_files(base) as sim:
            sim.write_xyz(path)
            X0 = sim.positions()
            sim.step(10)
            sim.write_xyz(path, append=True)
            X1 = sim.positions()
        frames = _read_xyz(path)
    assert len(frames) == 2
    assert frames[0][0].startswith("step 0 box") and frames[1][0].startswith("step 10 box")
    assert set(frames[0][1]) == {"Na", "Cl"}
    assert np.array_equal(frames[0][2], X0) and np.array_equal(frames[1][2], X1)


@pytest.mark.parametrize("kind", ["nacl_berendsen", "water_nh"])
def test_restart_continues_bit_for_bit(kind):
    """A restart read back by the context that wrote it and by a fresh
    context of the same system continues bit for bit alike (the file holds
    all the state), and within rounding of the uninterrupted run (reading
    rebuilds the list, which may reorder each row)."""
    with tempfile.TemporaryDirectory() as td:
        if kind == "nacl_berendsen":
            base = synth.write_case(synth.nacl_rocksalt(ncell=5, seed=62, nmaxlist=512), td, "s")
        else:
            base = synth.write_case(synth.water_grid(nside=9, seed=63), td, "s")
        rst = os.path.join(td, "run.rst")
        with MDSystem.from_files(base) as c:
            c.step(60)
            XC, hC = c.positions(), c.history(60)
        with MDSystem.from_files(base) as a:
            a.step(30)
            a.write_restart(rst)
            saved = a.thermo()
            Xs, Vs = a.positions(), a.velocities()
            a.read_restart(rst)
            a.step(30)
            XA, VA, hA = a.positions(), a.velocities(), a.history(30)
        with MDSystem.from_files(base) as b:
            b.read_restart(rst)
            assert np.array_equal(b.positions(), Xs)
            assert np.array_equal(b.velocities(), Vs)
            t = b.thermo()
            for k in ("temper", "lambda_", "xi"):
                assert t[k] == saved[k], k
            b.step(30)
            XB, VB, hB = b.positions(), b.velocities(), b.history(30)
        box = np.array([float(v) for v in open(base + ".cfg").read().split("\n")[1].split()])
    assert np.array_equal(XA, XB) and np.array_equal(VA, VB)
    assert [h["temper"] for h in hA] == [h["temper"] for h in hB]
    assert hB[-1]["step"] == hC[-1]["step"]
    d = XB - XC
    d -= box * np.rint(d / box)
    assert np.abs(d).max() <= 1e-3
    assert abs(hB[-1]["temper"] / hC[-1]["temper"] - 1) <= 1e-4
