"""Writes nacl64k_melt.npz: the starting state of the 64000-ion molten-NaCl
benchmark (LJ + Wolf, 1.5 g/cm^3), melted at 1200 K.

The rocksalt lattice of synth.nacl_rocksalt(ncell=20, seed=1) (0.25 A jitter,
Maxwell-Boltzmann velocities at 1200 K) is melted by this library's Berendsen
leapfrog on a GPU.  A defect-free lattice superheats (5 ps at 1200 K leave it
crystalline, 0.8 A rms from its sites), so it is first heated to 3000 K
(400 steps at dt 0.5 fs with tau 10 fs, then 2000 steps at dt 1 fs with tau
100 fs) and then brought to 1200 K (2500 steps, 5 ps, at dt 2 fs with tau
100 fs).  Positions and velocities are stored in FP32 in the input's atom
order (the reference's .cfg holds FP32 values), with the root-mean-square
displacement from the lattice sites as a record that the lattice melted.
Both arms of the benchmark (the library and the CPU restatement of the
reference's loop) start from this state.

    python -m md_gpu_gb300.cases.make_melt [output directory]     (needs a GPU)
"""
import os
import sys

import numpy as np

from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import synth
from md_gpu_gb300.replicas import equilibrate_batch

HERE = os.path.dirname(os.path.abspath(__file__))
HOT = (3000.0, ((0.5, 10.0, 400), (1.0, 100.0, 2000)))
COOL = (1200.0, ((2.0, 100.0, 2500),))


def main(out_dir=HERE):
    mdbuild.build()
    sys_ = synth.nacl_rocksalt(ncell=20, seed=1)
    a = synth.to_arrays(sys_)
    out = equilibrate_batch([a], temp=HOT[0], stages=HOT[1])
    out = equilibrate_batch(out, temp=COOL[0], stages=COOL[1])[0]
    pos = np.asarray(out["pos"], np.float32)
    vel = np.asarray(out["vel"], np.float32)
    L = np.asarray(sys_.box, np.float64)
    d = pos.astype(np.float64) - np.asarray(sys_.pos, np.float64)
    d -= L * np.rint(d / L)
    rmsd = float(np.sqrt((d * d).sum(1).mean()))
    np.savez_compressed(os.path.join(out_dir, "nacl64k_melt.npz"), pos=pos, vel=vel, ncell=20, seed=1,
                        rmsd_from_lattice=rmsd)
    print(f"nacl64k_melt.npz: {pos.shape[0]} ions, rms displacement from the lattice {rmsd:.2f} A")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
