"""The reference's own CUDA build, timed on the GPU beside the library.

The reference (md_gpu's src/) was written for CUDA 2.x and does not compile
with CUDA 13 as it stands: texture references were removed in CUDA 12, and
cudaMemcpyToSymbol no longer takes a symbol's name as a string.  prepare()
copies its sources, unmodified otherwise, into baseline/_ref/src (git-ignored;
the copy travels to the GPU machine with the repository) and applies a
mechanical three-part compat patch that keeps its arithmetic:

  1. forces.cu: the texture reference posTex becomes a __constant__ float4
     pointer, set by cudaMemcpyToSymbol where cudaBindTexture bound it;
  2. pair_forces.cu, bonded_forces.cu, energy.cu: tex1Dfetch(posTex, X)
     becomes posTex[X];
  3. neighborlist.cu, forces.cu, integrator.cu: cudaMemcpyToSymbol("name", ...)
     becomes cudaMemcpyToSymbol(::name, ...) (the file-scope __constant__;
     forces_init has locals of the same names, palfa and others, that would
     shadow it).

A fourth part repairs host heap overflows in its input parser, which glibc
on the GPU machine stops with an abort: simulation.cu zeroes 64 entries of
the 8-entry bond and angle parameter arrays (simulation.cu:211-229) and reads
the ensemble name and each atom-type name with %s into buffers of 3 and 2
bytes (simulation.cu:64,161).  Those four allocations get 64 entries and
LINE_LENGTH bytes; no value the reference computes changes.

build() compiles the eight translation units the reference's Makefile builds
besides athom.cu (src/Makefile:52) for sm_103a with the Makefile's -O3, plus
ref_driver.cu (a main program of this repository that calls the reference's
host entry points), into baseline/_ref/bin/ref_md.  It needs only nvcc, so it
runs on the GPU machine from the copied sources.

The reference's kernels check no bounds: neighborlist_nsquared writes up to
nmaxlist entries per atom without a test (neighborlist.cu:284) and
pair_forces* prefetch the entry after the last (pair_forces.cu:63,154).
check_case() therefore counts each atom's neighbours within rc + skin on the
host (the oracle's restatement of the same list) before any run and refuses
a case whose largest count is not well below nmaxlist.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
BIN = os.path.join(OUT, "bin", "ref_md")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
UNITS = ["gpu_properties.cu", "config.cu", "neighborlist.cu", "forces.cu", "integrator.cu", "runGPU.cu",
         "prints.cu", "simulation.cu"]
FLAGS = ["-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-w"]


def prepare(ref_src: str) -> bool:
    """Copy the reference's top-level sources and apply the compat patch;
    False when the reference tree is absent."""
    if not os.path.isdir(ref_src):
        return False
    os.makedirs(SRC, exist_ok=True)
    for f in sorted(os.listdir(ref_src)):
        p = os.path.join(ref_src, f)
        if os.path.isfile(p) and f.endswith((".cu", ".h")):
            shutil.copyfile(p, os.path.join(SRC, f))

    def patch(fname, fn):
        path = os.path.join(SRC, fname)
        with open(path) as fh:
            s = fh.read()
        t = fn(s)
        with open(path, "w") as fh:
            fh.write(t)
        return s != t

    tex = "texture<float4, 1, cudaReadModeElementType> posTex;"
    bind = "cudaBindTexture(0, posTex, g_conf->pos, sizeof(float4)*conf->natom);"

    def forces_fix(s):
        assert tex in s and bind in s, "forces.cu is not the expected version"
        s = s.replace(tex, "__constant__ float4 *posTex;")
        return s.replace(bind, "cudaMemcpyToSymbol(posTex, &g_conf->pos, sizeof(float4 *));")

    assert patch("forces.cu", forces_fix)
    for f in ("pair_forces.cu", "bonded_forces.cu", "energy.cu"):
        assert patch(f, lambda s: re.sub(r"tex1Dfetch\(\s*posTex\s*,\s*([^)]+)\)", r"posTex[\1]", s))
    for f in ("neighborlist.cu", "forces.cu", "integrator.cu"):
        patch(f, lambda s: re.sub(r'cudaMemcpyToSymbol\(\s*"(\w+)"', r"cudaMemcpyToSymbol( ::\1", s))

    def parser_fix(s):
        fixes = [("integ->ensemble = (char *)malloc(3);", "integ->ensemble = (char *)malloc(LINE_LENGTH);"),
                 ("fld->name[i] = (char *) malloc(2);", "fld->name[i] = (char *) malloc(LINE_LENGTH);")]
        for a in ("bnd1", "bnd2"):
            fixes.append((f"fld->{a} = (float *)malloc( nbo * sizeof(float) );",
                          f"fld->{a} = (float *)malloc( nbo * nbo * sizeof(float) );"))
        for a in ("ang1", "ang2"):
            fixes.append((f"fld->{a} = (float *)malloc( nag * sizeof(float) );",
                          f"fld->{a} = (float *)malloc( nag * nag * sizeof(float) );"))
        for old, new in fixes:
            assert old in s, "simulation.cu is not the expected version: " + old
            s = s.replace(old, new)
        return s

    assert patch("simulation.cu", parser_fix)
    return True


def have_sources() -> bool:
    return all(os.path.isfile(os.path.join(SRC, u)) for u in UNITS)


def build(force: bool = False) -> str:
    """Compile the patched sources and the driver (in parallel); returns the
    binary's path."""
    if not have_sources():
        raise RuntimeError("patched reference sources missing (baseline/_ref/src); run prepare() where "
                           "the reference tree exists")
    obj = os.path.join(OUT, "obj")
    os.makedirs(obj, exist_ok=True)
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    srcs = [os.path.join(SRC, u) for u in UNITS] + [os.path.join(HERE, "ref_driver.cu")]
    if not force and os.path.exists(BIN) and all(os.path.getmtime(BIN) > os.path.getmtime(s) for s in srcs):
        return BIN
    procs, objs = [], []
    for s in srcs:
        o = os.path.join(obj, os.path.basename(s).replace(".cu", ".o"))
        objs.append(o)
        procs.append((s, subprocess.Popen([NVCC] + FLAGS + ["-I", SRC, "-c", s, "-o", o],
                                          stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    bad = []
    for s, p in procs:
        out, _ = p.communicate()
        if p.returncode:
            bad.append(f"== {s}\n{out.decode(errors='replace')}")
    if bad:
        raise RuntimeError("reference build failed:\n" + "\n".join(bad))
    r = subprocess.run([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-o", BIN] + objs,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode:
        raise RuntimeError("reference link failed:\n" + r.stdout.decode(errors="replace"))
    return BIN


def check_case(base: str, margin: float = 1.3) -> int:
    """Largest neighbour count within rc + skin of the case's positions (the
    oracle's restatement of neighborlist_nsquared); raises unless
    margin * count + 1 <= nmaxlist, so that neither the list build nor the
    pair kernels' prefetch of the next entry can leave the list, and unless
    every atom has at most 3 bonds and 4 angles (the reference's per-atom
    bonded lists have 4 slots, filled unchecked, forces.cu:113-179, and
    bonded_forces prefetches the slot after an atom's last bond,
    bonded_forces.cu:54)."""
    import oracle
    case = oracle.load(base)
    p = case.params
    for arr, cols, lim in ((case.bonds, (1, 2), 3), (case.angles, (1, 2, 3), 4)):
        if len(arr):
            cnt = np.bincount(np.asarray(arr)[:, list(cols)].ravel(), minlength=case.natom)
            if cnt.max() > lim:
                raise ValueError(f"an atom is in more than {lim} bonded terms of one kind")
    excl = oracle.exclusions(case.natom, case.bonds)
    _, _, mx = oracle.nlist(case.pos4(), case.box, case.boxi, oracle.rskinsq(p.skin, p.rcutsq), excl,
                            p.nmaxlist)
    mx = int(mx)
    if margin * mx + 1 > p.nmaxlist:
        raise ValueError(f"largest neighbour count {mx} too close to nmaxlist {p.nmaxlist}")
    return mx


def _run(binary, mode, base, extra=(), timeout=900):
    d, name = os.path.dirname(base), os.path.basename(base)
    r = subprocess.run([binary, mode, name] + list(extra), cwd=d, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, timeout=timeout)
    out = r.stdout.decode(errors="replace")
    if r.returncode != 0 or "Cuda error" in out:
        raise RuntimeError(f"reference {mode} failed ({r.returncode}): {out[-2000:]}")
    return out


def forces(binary, base):
    """One list build and one force evaluation by the reference's kernels on
    the GPU, in the input's atom order: (list lengths, float4 forces, list
    columns nnlist[k, i] for k below the longest length)."""
    out = base + ".refforces"
    _run(binary, "forces", base, [out])
    with open(out, "rb") as fh:
        n = int(np.frombuffer(fh.read(4), np.int32)[0])
        nmax = np.frombuffer(fh.read(4 * n), np.uint32).copy()
        f4 = np.frombuffer(fh.read(16 * n), np.float32).reshape(n, 4).copy()
        pitch = int(np.frombuffer(fh.read(4), np.int32)[0])
        mx = int(np.frombuffer(fh.read(4), np.uint32)[0])
        cols = np.frombuffer(fh.read(4 * pitch * mx), np.uint32).reshape(mx, pitch)[:, :n].copy()
    os.unlink(out)
    return nmax, f4, cols


def write_timed_case(sys_, directory, nsteps):
    """The case with timrun = nsteps and a print interval beyond it (only
    step 0 prints, in every run)."""
    import dataclasses

    from md_gpu_gb300 import synth
    inp = dict(sys_.inp)
    t = inp["times"]
    inp["times"] = (t[0], int(nsteps), int(nsteps) + 1, t[3])
    return synth.write_case(dataclasses.replace(sys_, inp=inp), directory, "ref")


def time_steps(binary, sys_, tmp, nsteps, repeats=2):
    """Wall seconds of SimulationRun for nsteps steps less the same for 0
    steps (set-up, first list build and the one step t = 0), best of
    `repeats` each: seconds for nsteps MD steps of the reference's loop."""
    best = {}
    for k in (0, nsteps):
        base = write_timed_case(sys_, os.path.join(tmp, f"t{k}"), k)
        vals = []
        for _ in range(repeats):
            out = _run(binary, "run", base)
            m = re.search(r"REF_RUN_SECONDS ([0-9.eE+-]+)", out)
            vals.append(float(m.group(1)))
        best[k] = min(vals)
    return best[nsteps] - best[0], best
