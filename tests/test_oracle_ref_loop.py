"""The oracle's restatement of the reference's step loop run over consecutive
calls (md_ref_run_cont) equals one long call: the list built on the first call
persists, and later calls rebuild only on the displacement criterion, as the
reference's loop does between its steps (neighborlist.cu:109-146)."""
import numpy as np

import oracle
from md_gpu_gb300 import synth


def test_continued_loop_equals_one_run(tmp_path):
    case = oracle.load(synth.write_case(synth.nacl_rocksalt(ncell=4, seed=9), str(tmp_path), "n"))
    p1, v1 = case.pos4(), case.vel4()
    builds, _, _, t1 = oracle.md_ref_run(case, p1, v1, 24)
    p2, v2 = case.pos4(), case.vel4()
    st = oracle.RefLoopState(case.natom, case.params.nmaxlist)
    temper, total = None, 0
    for _ in range(3):
        b, temper = oracle.md_ref_run_cont(case, p2, v2, 8, st, temper=temper)
        total += b
    assert np.array_equal(p1, p2) and np.array_equal(v1, v2)
    assert total == builds and temper == t1
