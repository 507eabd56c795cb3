"""Energy drift of velocity-Verlet NVE, FP32 kernels against the FP64 mode of
the same library (md_set_precision 64) on the same seeded replicas: a smaller
version of the drift check bench.py makes on 16 replicas of 4000-atom argon.

6 replicas of 864-atom LJ argon (fcc 6^3 x 4, T* 0.72, dt 0.5 fs), 10 ps in
each precision.  The model (force truncated at rc) drifts by itself, so the
check is on the difference of the mean drifts: within 5 standard errors of
zero (a statistical check; the standard error at this size is ~1e-2
kT/atom/ns), and each precision's drift below 0.1 kT/atom/ns.
"""
import numpy as np
import pytest

from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import nve, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    mdbuild.build()


def test_fp32_drift_matches_fp64_drift():
    reps = [synth.to_arrays(synth.argon_fcc(ncell=6, seed=300 + r, integrator="vv")) for r in range(6)]
    natom = [len(a["itype"]) for a in reps]
    res = {}
    for prec in (32, 64):
        st, E = nve.energy_series(reps, 20000, 100, precision=prec)
        assert len(st) == 201 and st[-1] == 19901
        res[prec] = nve.drift(st, E, natom, 0.5, 0.72)
    m32, se32 = nve.summary(res[32])
    m64, se64 = nve.summary(res[64])
    se = float(np.hypot(se32, se64))
    print(f"drift FP32 {m32:.2e} +- {se32:.1e}, FP64 {m64:.2e} +- {se64:.1e} kT/atom/ns")
    assert abs(m32) < 0.1 and abs(m64) < 0.1
    assert abs(m32 - m64) <= 5 * se + 1e-4
