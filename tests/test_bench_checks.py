"""bench.py's FP64 checks (numpy / scipy: pair count, plain-form pair forces)
against the oracle."""
import importlib.util
import os

import numpy as np

import oracle
import golden_util as gu
from md_gpu_gb300 import synth

_spec = importlib.util.spec_from_file_location(
    "bench", os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py"))
bench = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(bench)


def test_pair_count_and_forces_match_oracle(tmp_path):
    case = oracle.load(synth.write_case(synth.nacl_rocksalt(ncell=4, seed=3), str(tmp_path), "n"))
    a = gu.case_arrays(case)
    pos = case.pos.astype(np.float64)
    rc = float(np.sqrt(a["rcutsq"]))
    pos4 = case.pos4()
    assert len(bench.pairs_within(pos, a["box"], rc)) == oracle.count_pairs(pos4, case.box, a["rcutsq"])
    nt = case.fld.ntype
    F, _ = bench.fp64_pair_forces(pos, a["box"], a["itype"], a["charge"], a["lj1"].reshape(nt, nt),
                                  a["lj2"].reshape(nt, nt), float(a["rcutsq"]), a["alfa"],
                                  bench.pairs_within(pos, a["box"], rc * 1.001))
    orc = gu.oracle_state(case)
    # the oracle takes some force-law constants as the reference's FP32
    # values; both are FP64 forms two orders below the 1e-5 gate they check
    assert gu.rms_rel(F, orc["f64"][:, :3]) <= 1e-7
