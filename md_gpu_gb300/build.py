"""Compile libmdgpu_gb300.so for sm_103a (nvcc, one process per translation
unit, in parallel).  Output: md_gpu_gb300/_build/libmdgpu_gb300.so."""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmdgpu_gb300.so")
SOURCES = ["md_api.cu", "k_cells.cu", "k_forces.cu", "k_integrate.cu", "k_probe.cu", "k_noalloc.cu", "k_fused.cu",
           "k_batch.cu", "k_adjoint.cu", "md_compat.cu", "k_pair64.cu", "k_pme.cu"]
HEADERS = ["md_internal.h", "md_device.cuh", "md_pair.cuh", "md_thermo.cuh",
           os.path.join("..", "..", "include", "md_gpu.h"), os.path.join("..", "..", "include", "md_gpu_compat.h")]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
# cuFFT (the PME transforms) is found there at run time as well
CUDA_LIB = os.path.join(os.path.dirname(os.path.dirname(NVCC)), "lib64")
# host code: no FMA contraction, so x86-64 (no FMA in its baseline) and
# aarch64 (FMA in its baseline) compute the same host-side constants
FLAGS = ["-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo",
         "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-Xcompiler", "-ffp-contract=off"]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    procs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, src):
            cmd = [NVCC] + FLAGS + ["-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd))
            procs.append((s, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for s, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((s, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(f"== {s}\n{o}" for s, o in failed))
    if force or procs or not os.path.exists(LIB):
        cmd = [NVCC, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB] + objs + \
              ["-lcufft", "-Xlinker", "-rpath", "-Xlinker", CUDA_LIB]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
