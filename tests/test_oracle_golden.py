"""The oracle against the golden vectors of the reference's own code.

Every FP32 array the oracle's "as written" mode produces must be byte-equal
to what the reference's kernels produced on the same inputs (hash compare);
the FP64 plain form must agree with them within FP32 rounding.
"""
import os
import tempfile

import numpy as np
import pytest

import oracle
import golden_util as gu

NAMES = gu.names()


@pytest.fixture(scope="module", params=NAMES)
def golden(request):
    g = gu.load_golden(request.param)
    case = gu.case_from_golden(g)
    return request.param, g, case


def _state(case, g):
    """Shared intermediate arrays recomputed with the oracle."""
    n = case.natom
    p = case.params
    pos4 = case.pos4()
    vel4 = case.vel4()
    excl = oracle.exclusions(n, case.bonds)
    rsk = oracle.rskinsq(p.skin, p.rcutsq)
    nn, nm, mx = oracle.nlist(pos4, case.box, case.boxi, rsk, excl, p.nmaxlist)
    wc = oracle.wolf_consts(p.alfa, p.rcutsq) if p.lkspace > 0 else np.zeros(4, np.float32)
    if p.lkspace != 1:
        wc[3] = 0.0
    kind = 0 if p.lkspace == 0 else 1
    reacf = p.reacf if p.lkspace == 0 else 0.0
    f = oracle.pair_f32(kind, pos4, case.box, case.boxi, nn, nm, case.fld.ntype, case.lj1,
                        case.lj2, p.rcutsq, reacf, wc)
    return dict(pos4=pos4, vel4=vel4, excl=excl, nn=nn, nm=nm, mx=mx, wc=wc, kind=kind,
                force_pair=f, rsk=rsk)


def test_parsed_inputs(golden):
    name, g, case = golden
    h = g["hashes"]
    n = case.natom
    assert gu.sha(case.itype) == h["itype"]
    pos_in = np.concatenate([case.pos, case.q[:, None]], 1).astype(np.float32)
    vel_in = np.concatenate([case.vel, case.mass[:, None]], 1).astype(np.float32)
    assert gu.sha(pos_in) == h["pos_in"]
    assert gu.sha(vel_in) == h["vel_in"]
    assert gu.sha(case.lj1) == h["lj1"]
    assert gu.sha(case.lj2) == h["lj2"]
    box = np.concatenate([case.box, case.boxi]).astype(np.float32)
    assert gu.sha(box) == h["box"]
    p = case.params
    pv = np.array([p.rcutsq, p.reacf, p.alfa, p.skin, p.nmaxlist, p.dt, p.temper_0, p.lkspace,
                   p.enstype, p.timrun, p.rdel, 0.0], np.float32)
    keep = [0, 2, 3, 4, 5, 6, 7, 8, 9, 10] + ([1] if p.lkspace == 0 else [])
    assert np.array_equal(pv[keep], g["params"][keep])
    for k in ("bnd1", "bnd2", "ang1", "ang2"):
        mine = np.ctypeslib.as_array(getattr(case.fld, k)).astype(np.float32)
        assert np.array_equal(mine[:8], g[k][:8]), k
    assert gu.sha(case.bonds.reshape(-1)) == h["bonds"]
    assert gu.sha(case.angles.reshape(-1)) == h["angles"]
    assert n == g["meta"]["natom"]


@pytest.mark.skipif(not os.path.isdir(gu.REF_ROOT), reason="reference example files absent")
def test_parser_on_reference_examples(golden):
    """The oracle's parser on the reference's example files equals the
    reference parser's result stored in the golden."""
    name, g, _ = golden
    if g["meta"]["kind"] != "example":
        pytest.skip("synthetic case")
    case = oracle.load(os.path.join(gu.REF_ROOT, g["meta"]["spec"]))
    pos_in = np.concatenate([case.pos, case.q[:, None]], 1).astype(np.float32)
    assert gu.sha(pos_in) == g["hashes"]["pos_in"]
    assert gu.sha(case.lj1) == g["hashes"]["lj1"]


def test_constants(golden):
    name, g, case = golden
    st = _state(case, g)
    c = g["consts"]
    p = case.params
    if p.lkspace > 0:
        wc = oracle.wolf_consts(p.alfa, p.rcutsq)
        if p.lkspace != 1:
            wc[3] = 0
        assert np.array_equal(wc, c[:4])
    assert st["rsk"] == c[4]
    assert oracle.rmaxdif(p.skin) == c[5]


def test_pack_and_exclusions(golden):
    name, g, case = golden
    st = _state(case, g)
    assert gu.sha(st["pos4"]) == g["hashes"]["pos4"]
    assert gu.sha(st["excl"]) == g["hashes"]["excl"]


def test_neighbour_list_bit_exact(golden):
    name, g, case = golden
    st = _state(case, g)
    n = case.natom
    assert np.array_equal(st["nm"][:n], g["nnlist_max"])
    rows = gu.rows_canonical(st["nn"], st["nm"], n, g["meta"]["list_width"])
    assert gu.sha(rows) == g["hashes"]["nnlist_rows"]


def test_neighbour_check(golden):
    name, g, case = golden
    st = _state(case, g)
    p = case.params
    rmd = oracle.rmaxdif(p.skin)
    pos4 = st["pos4"]
    half = np.sqrt(rmd, dtype=np.float32)
    p2 = pos4.copy()
    p2[case.natom // 2, 0] += np.float32(1.01) * half
    p3 = pos4.copy()
    p3[case.natom // 3, 1] += np.float32(0.99) * half
    got = [oracle.nlist_check(pos4, pos4, case.box, case.boxi, rmd),
           oracle.nlist_check(p2, pos4, case.box, case.boxi, rmd),
           oracle.nlist_check(p3, pos4, case.box, case.boxi, rmd)]
    assert got == list(g["nlist_check"])


def _forces(case, g, st):
    f = st["force_pair"].copy()
    out = {"force_pair": f.copy()}
    pt = oracle.pitch(case.natom)
    if len(case.bonds):
        bl, bm = oracle.bond_lists(case.natom, case.bonds, pt)
        oracle.bonds_f32(st["pos4"], case.box, case.boxi, bl, bm,
                         np.ctypeslib.as_array(case.fld.bnd1).astype(np.float32),
                         np.ctypeslib.as_array(case.fld.bnd2).astype(np.float32), f)
        out["force_bond"] = f.copy()
    if len(case.angles):
        al, am = oracle.angle_lists(case.natom, case.angles, pt)
        oracle.angles_f32(st["pos4"], case.box, case.boxi, al, am,
                          np.ctypeslib.as_array(case.fld.ang1).astype(np.float32),
                          np.ctypeslib.as_array(case.fld.ang2).astype(np.float32), f)
        out["force_angle"] = f.copy()
    out["force_total"] = f
    return out


def test_forces_bit_exact(golden):
    name, g, case = golden
    st = _state(case, g)
    for k, a in _forces(case, g, st).items():
        assert gu.sha(a) == g["hashes"][k], k


def test_integrators_bit_exact(golden):
    name, g, case = golden
    st = _state(case, g)
    f = _forces(case, g, st)["force_total"]
    p = case.params
    pos, vel = st["pos4"].copy(), st["vel4"].copy()
    oracle.leapfrog_nve_f32(pos, vel, f, p.dt, case.box, case.boxi)
    assert gu.sha(pos) == g["hashes"]["nve_pos"]
    assert gu.sha(vel) == g["hashes"]["nve_vel"]

    pos, vel = st["pos4"].copy(), st["vel4"].copy()
    scale = oracle.berendsen_scale(p.dt, np.float32(0.01), p.temper_0, np.float32(0.9) * np.float32(p.temper_0))
    assert np.float32(scale).tobytes() == g["nvt_scale"][:1].tobytes()
    part = oracle.leapfrog_nvt_f32(pos, vel, f, p.dt, scale, case.box, case.boxi)
    assert gu.sha(pos) == g["hashes"]["nvt_pos"]
    assert gu.sha(vel) == g["hashes"]["nvt_vel"]
    assert part.tobytes() == g["nvt_ke_partials"].tobytes()
    ks = oracle.ke_sum_ref(part)
    kt = np.array([ks * np.float32(0.5), oracle.temperature_ref(ks, case.natom)], np.float32)
    assert kt.tobytes() == g["nvt_ke_temper"].tobytes()

    pos, vel = st["pos4"].copy(), st["vel4"].copy()
    oracle.vv_pre_f32(pos, vel, f, p.dt, case.box, case.boxi)
    assert gu.sha(pos) == g["hashes"]["vvpre_pos"]
    assert gu.sha(vel) == g["hashes"]["vvpre_vel"]
    oracle.vv_cor_f32(vel, f, p.dt)
    assert gu.sha(vel) == g["hashes"]["vvcor_vel"]


def test_step_loop_bit_exact(golden):
    name, g, case = golden
    st = _state(case, g)
    nsteps = g["meta"]["nsteps"]
    pos, vel = st["pos4"].copy(), st["vel4"].copy()
    builds, f4, temps, _ = oracle.md_ref_run(case, pos, vel, nsteps)
    assert builds == int(g["run_builds"][0])
    assert gu.sha(pos) == g["hashes"]["run_pos"]
    assert gu.sha(vel) == g["hashes"]["run_vel"]
    assert gu.sha(f4) == g["hashes"]["run_force"]
    assert temps.tobytes() == g["run_temps"].tobytes()


def test_plain_form_close_to_reference(golden):
    """FP64 plain form vs the reference's FP32 pair forces (golden samples)."""
    name, g, case = golden
    st = _state(case, g)
    p = case.params
    f64, _ = oracle.pair_f64(st["kind"], st["pos4"], case.itype, case.q, case.box, st["nn"],
                             st["nm"], case.fld.ntype, case.lj1, case.lj2, p.rcutsq,
                             p.reacf if p.lkspace == 0 else 0.0, p.alfa)
    idx = g["sample_idx"]
    ref = g["sample__force_pair"].astype(np.float64)
    err = np.sqrt(((f64[idx, :3] - ref[:, :3]) ** 2).sum() / (f64[idx, :3] ** 2).sum())
    assert err < 2e-4, err
