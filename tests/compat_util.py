"""Helpers of the reference-compatible entry point tests: the C++ driver of
tests/compat (the reference's step loop through md_gpu_compat.h), its build
and its binary input/output."""
import os
import shutil
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER_SRC = os.path.join(ROOT, "tests", "compat", "compat_driver.cpp")
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")

# The reference's host entry points of the step loop (config.h:41-44,
# forces.h:44-50, neighborlist.h:40-42, integrator.h:50-56,
# gpu_properties.h:46-48), as demangled C++ signatures.
REFERENCE_SIGNATURES = [
    "gpu_properties_init(config*)",
    "gpu_properties_finish(gpu_struct*)",
    "checkCUDAError(char const*)",
    "config_init(config*)",
    "config_finish(config*, gpu_config*)",
    "config_HostToDevice(config*, gpu_config*)",
    "config_DeviceToHost(config*, gpu_config*, int)",
    "forces_init(ffield*, params*, config*, gpu_struct*, gpu_config*)",
    "forces(gpu_struct*, gpu_nlist*, gpu_config*, gpu_ffield*, ffield*, config*, params*)",
    "forces_finish(ffield*, gpu_ffield*)",
    "forces_HostToDevice(ffield*, gpu_ffield*)",
    "forces_DeviceToHost(ffield*, gpu_ffield*)",
    "energy(gpu_struct*, gpu_nlist*, gpu_config*, gpu_ffield*, ffield*, config*, params*)",
    "neighborlist_init(config*, gpu_struct*, params*, gpu_config*, ffield*)",
    "neighborlist(gpu_struct*, gpu_nlist*, gpu_config*, config*)",
    "neighborlist_finish(gpu_nlist*)",
    "integrate_init(integr*, gpu_struct*, config*)",
    "integrate_finish(integr*, gpu_integr*)",
    "integrate(gpu_config*, gpu_integr*, gpu_struct*, integr*, config*)",
    "integrate_pre(gpu_config*, gpu_integr*, gpu_struct*, integr*, config*)",
    "integrate_cor(gpu_config*, gpu_integr*, gpu_struct*, integr*, config*)",
    "integrate_HostToDevice(integr*, gpu_integr*, gpu_struct*)",
    "integrate_DeviceToHost(integr*, gpu_integr*, gpu_struct*)",
]


def build_driver(lib_path, out_dir):
    """Compile and link the driver against libmdgpu_gb300 (no GPU needed)."""
    exe = os.path.join(out_dir, "compat_driver")
    lib_dir = os.path.dirname(lib_path)
    cmd = [NVCC, "-std=c++17", "-O2", "-x", "cu", "-I", os.path.join(ROOT, "include"), DRIVER_SRC, "-o", exe,
           "-L", lib_dir, "-lmdgpu_gb300", "-Xlinker", "-rpath", "-Xlinker", lib_dir]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def write_input(path, a, nsteps, timprn):
    """The flat binary input of the driver from a to_arrays() system."""
    n, nt = len(a["itype"]), int(np.asarray(a["lj1"]).shape[0])
    with open(path, "wb") as f:
        np.array([n, nt, a["lkspace"], a["nmaxlist"], a["enstype"], nsteps, timprn], np.int32).tofile(f)
        np.array(list(a["box"]) + [a["rcutsq"], a["reacf"], a["alfa"], a["skin"], a["dt"], a["temper_0"]],
                 np.float32).tofile(f)
        np.asarray(a["itype"], np.int32).tofile(f)
        for k in ("charge", "pos", "vel", "type_mass", "lj1", "lj2"):
            np.asarray(a[k], np.float32).ravel().tofile(f)


def read_output(path, n, nsteps):
    d = np.fromfile(path, np.float32)
    pos = d[:3 * n].reshape(n, 3)
    vel = d[3 * n:6 * n].reshape(n, 3)
    temper = d[6 * n:6 * n + nsteps]
    q = d[6 * n + nsteps:6 * n + nsteps + n]
    return pos, vel, temper, q


def packed_charges(itype, q):
    """The charges the reference's kernels see: packed into pos.w by
    config_init (config.cu:34) and decoded as pair_forces.cu:44-45, in FP32."""
    t = np.asarray(itype).astype(np.float32)
    w = t + np.float32(0.1) * (np.asarray(q, np.float32) + np.float32(5.0))
    return (w - np.floor(w)) * np.float32(10.0) - np.float32(5.0)
