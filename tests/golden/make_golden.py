"""Generate the golden vectors that pin the oracle to the reference.

Runs oracle/_ref/ref_emu -- the reference's own .cfg/.fld/.inp parser
(simulation.cu) and kernel files (neighborlist.cu kernels, pair_forces.cu,
bonded_forces.cu, nve_leapfrog.cu, nvt_leapfrog_ber.cu, nve_vverlet.cu)
compiled unchanged as host C++ and executed on the CPU -- on a set of cases,
and stores per case an .npz with:

* the parsed inputs of reference example cases (the synthetic cases are
  regenerated from their seeds by md_gpu_gb300.synth at test time),
* the SHA-256 of every intermediate array the reference kernels produced
  (byte-exact FP32 results), plus small samples for diagnostics.

Usage (needs the reference tree; run in the build container):
    python tests/golden/make_golden.py [--ref <reference root>]   (default: $MD_GPU_REFERENCE)
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from md_gpu_gb300 import synth  # noqa: E402

# name -> (kind, spec, steps of the step-loop golden)
CASES = {
    "ex_h2o_wolf": ("example", "examples/h2o/wolf/h2o", 10),
    "ex_nacl_rf": ("example", "examples/nacl/nacl", 5),
    "syn_nacl_wolf": ("synth", {"fn": "nacl_rocksalt", "ncell": 8, "seed": 7, "nsteps": 20}, 20),
    "syn_water": ("synth", {"fn": "water_grid", "nside": 8, "seed": 11, "nsteps": 10,
                            "integrator": "leapfrog"}, 10),
    "syn_argon": ("synth", {"fn": "argon_fcc", "ncell": 6, "seed": 3, "nsteps": 20,
                            "integrator": "leapfrog"}, 20),
}

# arrays kept whole (small); everything else is stored as a hash + sample
KEEP = {"params", "fld_counts", "mass", "lj1", "lj2", "bnd1", "bnd2", "ang1", "ang2", "box",
        "consts", "nlist_check", "nvt_scale", "nvt_ke_temper", "nvt_ke_partials", "run_temps",
        "run_builds"}
INPUTS = {"itype", "pos_in", "vel_in", "bonds", "angles"}


def read_records(path):
    out = {}
    with open(path, "rb") as fh:
        while True:
            head = fh.read(64)
            if len(head) < 64:
                break
            name = head[:48].rstrip(b"\0").decode()
            dt = head[48:56].rstrip(b"\0").decode()
            count = int(np.frombuffer(head[56:64], np.uint64)[0])
            out[name] = np.frombuffer(fh.read(4 * count), np.dtype("<" + dt)).copy()
    return out


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def synth_case(spec, directory):
    spec = dict(spec)
    fn = getattr(synth, spec.pop("fn"))
    system = fn(**spec)
    return synth.write_case(system, directory, "case")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=oracle.REF_ROOT)
    args = ap.parse_args()
    exe = oracle.build_ref(os.path.join(args.ref, "src"))
    if exe is None:
        raise SystemExit("reference tree not found")
    index = {}
    for name, (kind, spec, nsteps) in CASES.items():
        with tempfile.TemporaryDirectory() as td:
            if kind == "example":
                base = os.path.join(args.ref, spec)
            else:
                base = synth_case(spec, td)
            out = os.path.join(td, "rec.bin")
            subprocess.run([exe, os.path.dirname(base), os.path.basename(base), out, str(nsteps)],
                           check=True)
            rec = read_records(out)
        store = {}
        hashes = {}
        n = int(rec["itype"].shape[0])
        rng = np.random.default_rng(0)
        sample = np.unique(np.concatenate([np.arange(min(16, n)), rng.integers(0, n, 16)]))
        store["sample_idx"] = sample.astype(np.int32)
        for k, a in rec.items():
            hashes[k] = sha(a)
            if k in KEEP or (kind == "example" and k in INPUTS):
                store[k] = a
            elif a.size >= 4 * n and a.size % n == 0 and k != "nnlist_rows":
                store["sample__" + k] = a.reshape(n, -1)[sample]
        rows = rec["nnlist_rows"]
        store["nnlist_max"] = rec["nnlist_max"]
        store["hashes"] = np.array(json.dumps(hashes))
        store["meta"] = np.array(json.dumps({"kind": kind, "spec": spec, "nsteps": nsteps,
                                             "natom": n, "list_width": int(rows.size // n)}))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **store)
        index[name] = {"kind": kind, "spec": spec, "nsteps": nsteps, "natom": n}
        print(name, n, "atoms,", len(hashes), "arrays")
    with open(os.path.join(HERE, "index.json"), "w") as fh:
        json.dump(index, fh, indent=1)


if __name__ == "__main__":
    main()
