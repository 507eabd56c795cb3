"""The C ABI without a GPU: the library loads, exports every entry point the
header declares, and rejects bad input on the host before any device work."""
import ctypes as C
import os
import re
import tempfile

import pytest

from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import synth
from md_gpu_gb300.system import MDError, MDSystem, library

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    mdbuild.build()
    return library()


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\s*(?:md_status|const char \*)\s*(md_\w+)\s*\(", text, re.M)
    return sorted(set(names))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_status_strings(lib):
    lib.md_status_string.restype = C.c_char_p
    assert lib.md_status_string(0) == b"ok"
    assert b"overflow" in lib.md_status_string(5)


def _case(tmp, **kw):
    return synth.write_case(synth.nacl_rocksalt(ncell=5, seed=1, **kw), tmp, "c")


def test_setters_reject_a_null_context(lib):
    """The reciprocal-sum, barostat and precision setters check their
    context before any device work."""
    lib.md_set_pme.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
    lib.md_set_barostat.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
    lib.md_set_precision.argtypes = [C.c_void_p, C.c_int]
    assert lib.md_set_pme(None, 32, 32, 32) == 1
    assert lib.md_set_barostat(None, 1.0, 1000.0, 4.5e-5) == 1
    assert lib.md_set_precision(None, 64) == 1


def test_missing_files(lib):
    with pytest.raises(MDError) as e:
        MDSystem.from_files("/nonexistent/run")
    assert e.value.status == 2


def test_malformed_inputs(lib):
    with tempfile.TemporaryDirectory() as tmp:
        base = _case(tmp)
        with open(base + ".cfg", "w") as fh:
            fh.write("12 1\n10.0 10.0\n")
        with pytest.raises(MDError) as e:
            MDSystem.from_files(base)
        assert e.value.status == 3
    with tempfile.TemporaryDirectory() as tmp:
        base = _case(tmp)
        with open(base + ".inp", "w") as fh:
            fh.write("ensemble: npt\ntemper: 300 1\n")   # the rest of the file is missing
        with pytest.raises(MDError) as e:
            MDSystem.from_files(base)
        assert e.value.status == 3
    with tempfile.TemporaryDirectory() as tmp:   # NPT runs the Berendsen leapfrog only
        base = synth.write_case(synth.nacl_rocksalt(ncell=5, seed=1, ensemble="npt", integrator="vv"), tmp, "c")
        with pytest.raises(MDError) as e:
            MDSystem.from_files(base)
        assert e.value.status == 7


def test_box_too_small_for_cutoff(lib):
    with tempfile.TemporaryDirectory() as tmp:
        base = synth.write_case(synth.nacl_rocksalt(ncell=4, seed=1), tmp, "c")   # L = 25.5 < 2 (rc + skin)
        with pytest.raises(MDError) as e:
            MDSystem.from_files(base)
        assert e.value.status == 8


def test_too_many_bonds(lib):
    with tempfile.TemporaryDirectory() as tmp:
        s = synth.water_grid(nside=8, seed=1)
        import numpy as np
        extra = np.array([[1, 1, 4], [1, 1, 5], [1, 1, 6]])   # atom 1 gets five bonds
        s.bonds = np.concatenate([s.bonds, extra])
        base = synth.write_case(s, tmp, "w")
        with pytest.raises(MDError) as e:
            MDSystem.from_files(base)
        assert e.value.status == 6


def test_batch_rejects_bad_replicas(lib):
    """md_create_batch validates every replica on the host: replicas must
    share dt / integrator and their bonded parameter tables (1), and each
    replica's cutoff + skin must fit half its box (8)."""
    import numpy as np
    a = synth.to_arrays(synth.nacl_replica(600, seed=1))
    b = synth.to_arrays(synth.nacl_replica(800, seed=2))
    bad_dt = dict(b, dt=1.0)
    with pytest.raises(MDError) as e:
        MDSystem.from_batch([a, bad_dt])
    assert e.value.status == 1
    small = dict(b, box=np.full(3, 20.0, np.float32))
    with pytest.raises(MDError) as e:
        MDSystem.from_batch([a, small])
    assert e.value.status == 8
    bonded = dict(b, bonds=np.array([[0, 0, 1]]), bnd1=[100.0], bnd2=[2.8])
    other = dict(a, bonds=np.array([[0, 0, 1]]), bnd1=[120.0], bnd2=[2.8])
    with pytest.raises(MDError) as e:
        MDSystem.from_batch([other, bonded])
    assert e.value.status == 1


def test_replica_batch_generator():
    """Uneven replica sizes in range, even, neutral; the cutoff is clamped so
    cutoff + skin fits half of every box."""
    import numpy as np
    reps = synth.replica_batch(24, seed=5)
    sizes = [r.natom for r in reps]
    assert min(sizes) >= 256 and max(sizes) <= 8192 and all(n % 2 == 0 for n in sizes)
    assert len(set(sizes)) > 12
    for r in reps:
        rc = r.inp["cutoff"][0]
        assert 2 * (rc + r.inp["skin"][0]) < r.box[0]
        assert abs(r.charge.sum()) < 1e-9
        assert np.all(np.abs(r.pos) <= 0.5 * r.box[0])
    small = synth.nacl_replica(256, seed=1)
    assert small.inp["cutoff"][0] < 12.0
