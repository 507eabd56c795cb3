"""Failure paths of the CUDA path, made without faulting the GPU.

* A grid barrier of the one-kernel list rebuild whose wait runs out: a test
  hook makes one block of the rebuild leave before the first barrier and
  shortens the wait to 2 ms.  Every other block gives up after 2 ms, sets the
  sticky status and returns; no later phase runs (the atom order and the
  build count are unchanged), later rebuilds return at once, the calls
  report the timeout, and a new context on the same CUDA context runs
  normally.
"""
import tempfile

import numpy as np
import pytest

from md_gpu_gb300 import MDSystem
from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import synth
from md_gpu_gb300.system import MDError, library

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    mdbuild.build()


def _nacl(td, ncell=6, seed=3, **kw):
    return synth.write_case(synth.nacl_rocksalt(ncell=ncell, seed=seed, **kw), td, "f")


def test_rebuild_barrier_timeout_stops_the_rebuild():
    with tempfile.TemporaryDirectory() as td:
        base = _nacl(td)
        sim = MDSystem.from_files(base)
        try:
            sim.set_tuning(8, 0)        # warp-per-cell builder: the one-kernel rebuild
            sim.step(4)
            info0 = sim.info()
            order0 = sim.order()
            L = library()
            assert L.md_debug_rebuild_barrier(sim._ctx, 2.0, 0) == 0
            with pytest.raises(MDError) as e:
                sim.update_neighbors(force=True)
            assert e.value.status == 4 and "grid barrier" in str(e.value)
            # nothing after the first barrier ran: same order, same build count
            info1 = sim.info()
            assert info1["builds"] == info0["builds"]
            assert np.array_equal(sim.order(), order0)
            # the error is sticky: later rebuilds do nothing and steps report it
            with pytest.raises(MDError) as e2:
                sim.step(40)
            assert "grid barrier" in str(e2.value)
            assert sim.info()["builds"] == info0["builds"]
        finally:
            sim.close()
        # the CUDA context is intact: a new context on the same files runs
        with MDSystem.from_files(base) as sim2:
            sim2.set_tuning(8, 0)
            sim2.step(16)
            t = sim2.thermo()
            assert t["step"] == 15 and np.isfinite(t["temper"]) and t["temper"] > 0
