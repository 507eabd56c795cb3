"""The reference-compatible entry points (include/md_gpu_compat.h) without a
GPU: the library exports each of the reference's step-loop functions under
its C++ signature, and a program written against them (the reference's loop,
tests/compat/compat_driver.cpp) compiles and links."""
import os
import shutil
import subprocess
import tempfile

import pytest

import compat_util as cu
import oracle
from md_gpu_gb300 import build as mdbuild


@pytest.fixture(scope="module")
def lib_path():
    return mdbuild.build()


def test_reference_signatures_exported(lib_path):
    nm = shutil.which("nm")
    if not nm:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-DC", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = {line.split(" ", 2)[2].strip() for line in out.splitlines() if line.count(" ") >= 2}
    for sig in cu.REFERENCE_SIGNATURES:
        assert sig in exported, sig


def test_reference_loop_links(lib_path):
    if not os.path.exists(cu.NVCC):
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as td:
        exe = cu.build_driver(lib_path, td)
        assert os.path.exists(exe)


REF_SRC = oracle.REF_SRC


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not present")
def test_reference_main_program_links(lib_path):
    """The reference's own athom.cu, runGPU.cu, simulation.cu and prints.cu,
    unmodified, link against the library (tests/compat/Makefile)."""
    if not os.path.exists(cu.NVCC):
        pytest.skip("nvcc not available")
    here = os.path.join(cu.ROOT, "tests", "compat")
    out = os.path.join(cu.ROOT, "oracle", "_ref", "athom_md")
    if os.path.exists(out):
        os.unlink(out)
    r = subprocess.run(["make", "-s", "-C", here, "ref-main", f"NVCC={cu.NVCC}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    assert os.path.exists(out)
