"""md_ref_kinetic_energy_noalloc: the kinetic energy / temperature entry point
for callers that cannot let a library allocate device memory (it keeps its
partial sums in a fixed __device__ array).  Checked through the C ABI against
the context path (md_get_thermo, whose reduction uses allocated scratch) on
the same velocities, on two calls in a row.  Collected last on purpose."""
import ctypes as C
import tempfile

import numpy as np
import pytest

import oracle
from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import synth
from md_gpu_gb300.system import MDSystem, library

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12     # both sides are FP64 sums of the same FP64 terms


def test_noalloc_kinetic_energy_matches_context_path():
    torch = pytest.importorskip("torch")
    mdbuild.build()
    L = library()
    with tempfile.TemporaryDirectory() as td:
        base = synth.write_case(synth.nacl_rocksalt(ncell=6, seed=17), td, "ke")
        case = oracle.load(base)
        with MDSystem.from_files(base) as sim:
            th = sim.thermo()
    vel4 = np.ascontiguousarray(np.concatenate([case.vel, case.mass[:, None]], 1), np.float32)
    d_vel = torch.from_numpy(vel4).cuda()
    d_out = torch.zeros(2, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        d_out.zero_()
        torch.cuda.synchronize()
        st = L.md_ref_kinetic_energy_noalloc(C.c_void_p(d_vel.data_ptr()), case.natom,
                                              C.c_void_p(d_out.data_ptr()), None)
        assert st == 0
        ke, temper = d_out.cpu().numpy()
        assert abs(ke - th["ke"]) <= REL_TOL * abs(th["ke"])
        assert abs(temper - th["temper"]) <= REL_TOL * abs(th["temper"])


def test_noalloc_allocates_nothing_and_runs_on_any_stream():
    """After the first call (which loads the kernels), further calls leave the
    device's free memory unchanged, also on a stream other than the default."""
    torch = pytest.importorskip("torch")
    mdbuild.build()
    L = library()
    rng = np.random.default_rng(5)
    n = 50000
    vel4 = np.empty((n, 4), np.float32)
    vel4[:, :3] = rng.normal(0.0, 0.01, (n, 3))
    vel4[:, 3] = 230000.0
    d_vel = torch.from_numpy(vel4).cuda()
    d_out = torch.zeros(2, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    assert L.md_ref_kinetic_energy_noalloc(C.c_void_p(d_vel.data_ptr()), n, C.c_void_p(d_out.data_ptr()),
                                           None) == 0
    torch.cuda.synchronize()
    ref = d_out.cpu().numpy().copy()
    free0, _ = torch.cuda.mem_get_info()
    for k in range(6):
        stream = C.c_void_p(s.cuda_stream) if k % 2 else None
        assert L.md_ref_kinetic_energy_noalloc(C.c_void_p(d_vel.data_ptr()), n,
                                               C.c_void_p(d_out.data_ptr()), stream) == 0
        torch.cuda.synchronize()
        assert np.array_equal(d_out.cpu().numpy(), ref)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    ke64 = 0.5 * (vel4[:, 3].astype(np.float64) * (vel4[:, :3].astype(np.float64) ** 2).sum(1)).sum()
    assert abs(ref[0] - ke64) <= 1e-12 * ke64


def test_noalloc_rejects_sizes_beyond_its_scratch():
    library()
    L = library()
    st = L.md_ref_kinetic_energy_noalloc(C.c_void_p(16), 1048577, C.c_void_p(16), None)
    assert st == 1
    buf = C.create_string_buffer(256)
    L.md_last_error(None, buf, 256)
    assert b"exceeds" in buf.value
