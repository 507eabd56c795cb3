"""CUDA path vs the oracle, through the C ABI (libmdgpu_gb300.so).

Tolerances (stated, per the path's precision contract):
* neighbour lists: bit-exact as sets and as sorted rows (integer work);
* forces: RMS relative error <= 1e-5 against the FP64 plain form
  (sqrt(sum |F - F64|^2 / sum |F64|^2)), same Coulomb model (A&S 7.1.26);
* energies: RMS relative <= 2e-5 per atom, 1e-6 on totals;
* one integrator step: velocity increments RMS relative <= 2e-5, positions
  to 1e-6 A.
"""
import os
import tempfile

import numpy as np
import pytest

import oracle
import golden_util as gu
from md_gpu_gb300 import MD_LEAPFROG, MD_NH, MD_VV, TERM_ALL, TERM_ANGLE, TERM_BOND, TERM_PAIR
from md_gpu_gb300 import build as mdbuild
from md_gpu_gb300 import synth

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _lib():
    mdbuild.build()


@pytest.fixture(scope="module", params=gu.names())
def gcase(request):
    g = gu.load_golden(request.param)
    case = gu.case_from_golden(g)
    return request.param, g, case


def test_neighbour_list_bit_exact(gcase):
    name, g, case = gcase
    orc = gu.oracle_state(case)
    with gu.system_from_case(case) as sim:
        width = g["meta"]["list_width"]
        nn, nm = sim.neighbor_list(width)
        n = case.natom
        assert np.array_equal(nm[:n], orc["nm"][:n])
        rows = gu.rows_canonical(nn, nm, n, width)
        assert np.array_equal(rows, gu.rows_canonical(orc["nn"], orc["nm"], n, width))
        assert gu.sha(rows) == g["hashes"]["nnlist_rows"]


def test_pair_forces_vs_fp64(gcase):
    name, g, case = gcase
    orc = gu.oracle_state(case)
    with gu.system_from_case(case) as sim:
        sim.compute_forces(TERM_PAIR)
        F = sim.forces()
    err = gu.rms_rel(F[:, :3], orc["f64"][:, :3])
    assert err <= FORCE_TOL, err
    assert gu.rms_rel(F[:, 3], orc["f64"][:, 3]) <= FORCE_TOL


def test_pair_forces_vs_reference_kernel(gcase):
    """Against the reference kernel's own FP32 result (golden samples)."""
    name, g, case = gcase
    with gu.system_from_case(case) as sim:
        sim.compute_forces(TERM_PAIR)
        F = sim.forces()
    idx = g["sample_idx"]
    ref = g["sample__force_pair"].astype(np.float64)
    assert gu.rms_rel(F[idx, :3], ref[:, :3]) <= 2 * FORCE_TOL


def test_energies_vs_fp64(gcase):
    name, g, case = gcase
    orc = gu.oracle_state(case)
    with gu.system_from_case(case) as sim:
        sim.compute_forces(TERM_PAIR, energy=True)
        ep = sim.energies()
        th = sim.thermo()
    assert gu.rms_rel(ep, orc["ep64"]) <= 2e-5
    assert abs(th["pe"] - orc["ep64"].sum()) <= 1e-6 * np.abs(orc["ep64"]).sum()


def test_bonded_forces_vs_fp64(gcase):
    name, g, case = gcase
    if not len(case.bonds) and not len(case.angles):
        pytest.skip("no bonded terms")
    pos4 = case.pos4()
    f = np.zeros((case.natom, 4))
    ep = np.zeros(case.natom)
    arr = lambda k: np.ctypeslib.as_array(getattr(case.fld, k)).astype(np.float32)
    if len(case.bonds):
        oracle.bonds_f64(pos4, case.box, case.bonds, arr("bnd1"), arr("bnd2"), f, ep)
    if len(case.angles):
        oracle.angles_f64(pos4, case.box, case.angles, arr("ang1"), arr("ang2"), f, ep)
    with gu.system_from_case(case) as sim:
        sim.compute_forces(TERM_BOND | TERM_ANGLE, energy=True)
        F = sim.forces()
        E = sim.energies()
    assert gu.rms_rel(F[:, :3], f[:, :3]) <= FORCE_TOL
    assert gu.rms_rel(E, ep) <= 2e-5


def test_total_forces(gcase):
    name, g, case = gcase
    orc = gu.oracle_state(case)
    f = orc["f64"].copy()
    ep = np.zeros(case.natom)
    arr = lambda k: np.ctypeslib.as_array(getattr(case.fld, k)).astype(np.float32)
    pos4 = orc["pos4"]
    if len(case.bonds):
        oracle.bonds_f64(pos4, case.box, case.bonds, arr("bnd1"), arr("bnd2"), f, ep)
    if len(case.angles):
        oracle.angles_f64(pos4, case.box, case.angles, arr("ang1"), arr("ang2"), f, ep)
    with gu.system_from_case(case) as sim:
        sim.compute_forces(TERM_ALL)
        F = sim.forces()
    assert gu.rms_rel(F[:, :3], f[:, :3]) <= FORCE_TOL


def test_leapfrog_one_step(gcase):
    name, g, case = gcase
    orc = gu.oracle_state(case)
    f = orc["f64"][:, :3].copy()
    arr = lambda k: np.ctypeslib.as_array(getattr(case.fld, k)).astype(np.float32)
    f4 = np.zeros((case.natom, 4))
    ep = np.zeros(case.natom)
    if len(case.bonds):
        oracle.bonds_f64(orc["pos4"], case.box, case.bonds, arr("bnd1"), arr("bnd2"), f4, ep)
    if len(case.angles):
        oracle.angles_f64(orc["pos4"], case.box, case.angles, arr("ang1"), arr("ang2"), f4, ep)
    f += f4[:, :3]
    p = case.params
    m = case.mass.astype(np.float64)
    x0 = case.pos.astype(np.float64)
    v0 = case.vel.astype(np.float64)
    v1 = v0 + f * p.dt / m[:, None]          # first Berendsen step has lambda = 1
    x1 = x0 + v1 * p.dt
    L = case.box.astype(np.float64)
    x1 -= L * np.trunc(x1 * 2.0 / L)
    with gu.system_from_case(case, integrator=MD_LEAPFROG) as sim:
        sim.step(1)
        X, V = sim.positions(), sim.velocities()
    assert gu.rms_rel(V - v0, v1 - v0) <= 2e-5
    assert np.abs(X - x1).max() <= 1e-6 * max(1.0, float(L.max()))


def test_determinism():
    case = oracle.load(_write(synth.nacl_rocksalt(ncell=6, seed=5)))
    outs = []
    for _ in range(2):
        with gu.system_from_case(case) as sim:
            sim.step(40)
            outs.append((sim.positions(), sim.velocities(), sim.forces(), sim.thermo()["temper"]))
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(np.asarray(a), np.asarray(b))


_TMP = tempfile.mkdtemp(prefix="mdgpu_")


def _write(system, name="case"):
    d = tempfile.mkdtemp(dir=_TMP)
    return synth.write_case(system, d, name)


def test_files_and_arrays_agree():
    base = _write(synth.water_grid(nside=8, seed=2))
    case = oracle.load(base)
    from md_gpu_gb300 import MDSystem
    with MDSystem.from_files(base) as a, gu.system_from_case(case) as b:
        a.compute_forces()
        b.compute_forces()
        assert np.array_equal(a.forces(), b.forces())
        assert np.array_equal(a.positions(), b.positions())


def test_cell_order_is_hilbert_sorted():
    case = oracle.load(_write(synth.nacl_rocksalt(ncell=6, seed=9)))
    p = case.params
    rl = np.float32(np.sqrt(np.float32(p.rcutsq))) + np.float32(p.skin)
    nc, bl = oracle.cell_dims(case.box, rl)
    with gu.system_from_case(case) as sim:
        info = sim.info()
        assert list(nc) == info["ncell"]
        assert np.array_equal(bl, np.array(info["binlen"], np.float32))
        ranks = sim.cell_ranks()
        bits = max(1, int(np.ceil(np.log2(max(nc)))))
        keys = []
        for z in range(nc[2]):
            for y in range(nc[1]):
                for x in range(nc[0]):
                    keys.append((oracle.hilbert3(x, y, z, bits), x + nc[0] * (y + nc[1] * z)))
        expect = np.zeros(len(keys), np.int32)
        for r, (_, lin) in enumerate(sorted(keys)):
            expect[lin] = r
        assert np.array_equal(ranks, expect)
        cell = oracle.cell_index(case.pos4(), case.box, nc, bl)
        lin = cell[:, 0] + nc[0] * (cell[:, 1] + nc[1] * cell[:, 2])
        expect_order = np.lexsort((np.arange(case.natom), expect[lin]))
        assert np.array_equal(sim.order(), expect_order)


def test_berendsen_temperatures_vs_plain():
    case = oracle.load(_write(synth.nacl_rocksalt(ncell=5, seed=3, nmaxlist=512)))
    x = case.pos.astype(np.float64).copy()
    v = case.vel.astype(np.float64).copy()
    st, rec = oracle.md_plain_run(case, x, v, 5, 0)
    with gu.system_from_case(case, integrator=MD_LEAPFROG) as sim:
        sim.step(5)
        hist = sim.history(5)
        X = sim.positions()
    t_gpu = np.array([h["temper"] for h in hist])
    t_orc = 2.0 * rec[:, 0] / ((3 * case.natom - 3) * 8.314e-3)
    assert np.abs(t_gpu / t_orc - 1).max() <= 1e-5
    d = X - x
    L = case.box.astype(np.float64)
    d -= L * np.rint(d / L)
    assert np.abs(d).max() <= 1e-4


def test_velocity_verlet_energy_and_plain_form():
    case = oracle.load(_write(synth.argon_fcc(ncell=5, seed=4, integrator="vv")))
    x = case.pos.astype(np.float64).copy()
    v = case.vel.astype(np.float64).copy()
    st, rec = oracle.md_plain_run(case, x, v, 50, 1)
    with gu.system_from_case(case, integrator=MD_VV) as sim:
        sim.step(50, energy_every=1)
        hist = sim.history(50)
    ke = np.array([h["ke"] for h in hist])
    pe = np.array([h["pe"] for h in hist])
    assert np.abs(ke - rec[:, 0]).max() <= 1e-4 * np.abs(rec[:, 0]).max()
    assert np.abs(pe - rec[:, 1]).max() <= 1e-4 * np.abs(rec[:, 1]).max()
    e = ke + pe
    assert np.ptp(e) <= 5e-3 * np.abs(pe).mean()


def test_nose_hoover_conserved():
    case = oracle.load(_write(synth.water_grid(nside=8, seed=8, integrator="nh", dt=0.5)))
    x = case.pos.astype(np.float64).copy()
    v = case.vel.astype(np.float64).copy()
    st, rec = oracle.md_plain_run(case, x, v, 20, 2)
    with gu.system_from_case(case, integrator=MD_NH) as sim:
        sim.step(20, energy_every=1)
        hist = sim.history(20)
    cons = np.array([h["conserved"] for h in hist])
    ke = np.array([h["ke"] for h in hist])
    assert np.abs(ke - rec[:, 0]).max() <= 1e-4 * np.abs(rec[:, 0]).max()
    assert np.abs(cons - rec[:, 2]).max() <= 1e-4 * np.abs(rec[:, 2]).max()
    assert np.abs(np.array([h["xi"] for h in hist])).max() > 0


def test_run_host_matches_step():
    case = oracle.load(_write(synth.nacl_rocksalt(ncell=5, seed=12, nmaxlist=512)))
    with gu.system_from_case(case) as a, gu.system_from_case(case) as b:
        p0, v0 = a.positions(), a.velocities()
        p, v, recs = a.run_host(p0, v0, 12)
        b.step(12)
        assert np.array_equal(p, b.positions())
        assert np.array_equal(v, b.velocities())
        assert [r["temper"] for r in recs] == [h["temper"] for h in b.history(12)]
    # in place from pinned-style buffers, records as a structured array
    with gu.system_from_case(case) as c:
        hp, hv = np.ascontiguousarray(p0), np.ascontiguousarray(v0)
        out_p, out_v, raw = c.run_host(hp, hv, 12, inplace=True, raw_records=True)
        assert out_p is hp and out_v is hv
        assert np.array_equal(hp, p) and np.array_equal(hv, v)
        assert list(raw["temper"]) == [r["temper"] for r in recs]


def test_list_rebuilds_keep_parity():
    """After many steps (several rebuilds and re-sorts) the list is still the
    O(N^2) reference list of the current positions."""
    case = oracle.load(_write(synth.nacl_rocksalt(ncell=5, seed=21, nmaxlist=512)))
    with gu.system_from_case(case) as sim:
        sim.step(60)
        info = sim.info()
        assert info["builds"] >= 2
        pos = sim.positions().astype(np.float32)
        # the list was built at the last rebuild; rebuild now at the current positions
        sim.update_neighbors(force=True)
        nn, nm = sim.neighbor_list(512)
    q = case.q
    pos4 = np.concatenate([pos, (case.itype.astype(np.float32) + np.float32(0.1) * (q + np.float32(5.0)))[:, None]], 1)
    pos4 = np.ascontiguousarray(pos4, np.float32)
    p = case.params
    onn, onm, _ = oracle.nlist(pos4, case.box, case.boxi, oracle.rskinsq(p.skin, p.rcutsq),
                               oracle.exclusions(case.natom, case.bonds), 512)
    n = case.natom
    assert np.array_equal(nm[:n], onm[:n])
    assert np.array_equal(gu.rows_canonical(nn, nm, n, 512), gu.rows_canonical(onn, onm, n, 512))


def _tie_lattice(seed, jitter=4e-6):
    """Simple-cubic lattice of spacing rl/5 (8000 sites, box 4 rl): every site
    has 30 lattice neighbours at exactly rl (vectors (5,0,0) and (3,4,0)
    and their permutations), and the jitter of a few ulps puts the FP32 r^2
    of each such pair within a few ulps of rl^2 on either side."""
    s = synth.nacl_rocksalt(ncell=5, seed=seed, nmaxlist=640)
    a, m = 13.0 / 5.0, 20
    g = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)
    L = a * m
    rng = np.random.default_rng(seed)
    s.box = np.full(3, L)
    s.pos = g * a - 0.5 * L + 0.3 + rng.uniform(-jitter, jitter, g.shape)
    s.itype = np.where(g.sum(1) % 2 == 0, 1, 2).astype(np.int64)
    s.charge = np.where(s.itype == 1, 1.0, -1.0)
    s.vel = np.zeros_like(s.pos)
    return s


@pytest.mark.parametrize("list_tpa", [0, 8])
def test_list_threshold_ties(list_tpa):
    """Pairs whose FP32 r^2 lies within a few ulps of (rc + skin)^2 (30 per
    atom here): the list predicate rounds every operation exactly as the
    reference writes it, so the list equals the oracle's bit for bit, for the
    list built at creation and for a rebuild after new positions."""
    case = oracle.load(_write(_tie_lattice(seed=3)))
    assert case.params.skin == 1.0 and np.float32(case.params.rcutsq) == np.float32(144.0)
    p = case.params
    n = case.natom
    with gu.system_from_case(case) as sim:
        sim.set_tuning(8, list_tpa)
        sim.update_neighbors(force=True)
        nn, nm = sim.neighbor_list(640)
        orc = gu.oracle_state(case)
        assert np.array_equal(nm[:n], orc["nm"][:n])
        assert np.array_equal(gu.rows_canonical(nn, nm, n, 640), gu.rows_canonical(orc["nn"], orc["nm"], n, 640))
        # 484 lattice neighbours lie strictly inside rl; of the 30 ties about
        # half are in, so the ties are really decided by rounding
        assert (484 + 6) * n < int(orc["nm"][:n].sum()) < (484 + 24) * n
        x2 = _tie_lattice(seed=4).pos
        sim.set_positions(x2)
        sim.update_neighbors(force=True)
        nn, nm = sim.neighbor_list(640)
    pos4 = case.pos4().copy()
    pos4[:, :3] = x2.astype(np.float32)
    onn, onm, _ = oracle.nlist(pos4, case.box, case.boxi, oracle.rskinsq(p.skin, p.rcutsq),
                               oracle.exclusions(n, case.bonds), 640)
    assert np.array_equal(gu.rows_canonical(nn, nm, n, 640), gu.rows_canonical(onn, onm, n, 640))


@pytest.mark.parametrize("pair_tpa,list_tpa,depth", [(1, 1, 0), (2, 0, 0), (4, 4, 4), (8, 8, 0),
                                                     (8, 0, 2), (16, 0, 0), (16, 16, 1), (32, 32, 0)])
def test_thread_split_variants(pair_tpa, list_tpa, depth):
    case = oracle.load(_write(synth.nacl_rocksalt(ncell=5, seed=30, nmaxlist=512)))
    orc = gu.oracle_state(case)
    with gu.system_from_case(case) as sim:
        sim.set_tuning(pair_tpa, list_tpa, depth)
        assert sim.info()["pair_depth"] == (depth or {1: 8, 2: 8, 4: 8, 8: 4, 16: 2, 32: 1}[pair_tpa])
        sim.update_neighbors(force=True)
        sim.compute_forces(TERM_PAIR, energy=True)
        F = sim.forces()
        E = sim.energies()
        nn, nm = sim.neighbor_list(512)
    assert gu.rms_rel(F[:, :3], orc["f64"][:, :3]) <= FORCE_TOL
    assert gu.rms_rel(E, orc["ep64"]) <= 2e-5
    n = case.natom
    assert np.array_equal(gu.rows_canonical(nn, nm, n, 512), gu.rows_canonical(orc["nn"], orc["nm"], n, 512))


def test_positions_outside_the_box():
    """Positions given in [0, L) instead of [-L/2, L/2] (the reference takes
    either: its list is all pairs with the minimum-image shift).  Cells then
    bin the periodic images and every pair takes the shift; the list stays
    bit-exact and the forces within tolerance.  Centred input turns the fast
    paths back on."""
    case = oracle.load(_write(synth.nacl_rocksalt(ncell=10, seed=31, nmaxlist=512)))
    L = case.box.astype(np.float64)
    with gu.system_from_case(case) as sim:
        assert sim.info()["centered"]
        X = sim.positions()
        sim.compute_forces(TERM_PAIR)
        F0 = sim.forces()
        moved = np.where(X < 0, X + L, X)
        sim.set_positions(moved)
        assert not sim.info()["centered"]
        sim.compute_forces(TERM_PAIR)
        F1 = sim.forces()
        nn, nm = sim.neighbor_list(512)
        sim.step(40)                       # the integrator wraps x >= L/2 back
        sim.set_positions(X)
        assert sim.info()["centered"]
    pos4 = case.pos4().copy()
    pos4[:, :3] = moved.astype(np.float32)
    p = case.params
    onn, onm, _ = oracle.nlist(pos4, case.box, case.boxi, oracle.rskinsq(p.skin, p.rcutsq),
                               oracle.exclusions(case.natom, case.bonds), 512)
    n = case.natom
    assert np.array_equal(nm[:n], onm[:n])
    assert np.array_equal(gu.rows_canonical(nn, nm, n, 512), gu.rows_canonical(onn, onm, n, 512))
    orc = gu.oracle_state(case)
    assert gu.rms_rel(F1[:, :3], orc["f64"][:, :3]) <= FORCE_TOL
    assert gu.rms_rel(F1[:, :3], F0[:, :3]) <= FORCE_TOL


def test_full_size_nacl_64k():
    """The 64000-ion system: bit-exact list, forces within tolerance, and
    size-independent properties (momentum, Newton's third law in sum)."""
    base = _write(synth.nacl_rocksalt(ncell=20, seed=1), "nacl64k")
    case = oracle.load(base)
    orc = gu.oracle_state(case)
    from md_gpu_gb300 import MDSystem
    with MDSystem.from_files(base) as sim:
        nn, nm = sim.neighbor_list(512)
        sim.compute_forces(TERM_PAIR)
        F = sim.forces()
    n = case.natom
    assert np.array_equal(nm[:n], orc["nm"][:n])
    assert np.array_equal(gu.rows_canonical(nn, nm, n, 512), gu.rows_canonical(orc["nn"], orc["nm"], n, 512))
    assert gu.rms_rel(F[:, :3], orc["f64"][:, :3]) <= FORCE_TOL
    assert np.abs(F[:, :3].sum(0)).max() <= 1e-3 * np.sqrt((F[:, :3] ** 2).sum(1)).mean() * np.sqrt(n)


def test_type_exclusions():
    """Excluding every O-H pair by type removes exactly those pairs from the
    reference list."""
    case = oracle.load(_write(synth.water_grid(nside=8, seed=4)))
    orc = gu.oracle_state(case)
    n = case.natom
    with gu.system_from_case(case) as sim:
        sim.set_type_exclusions(np.array([1 << 1, 0], np.uint32))
        nn, nm = sim.neighbor_list(768)
    rows = oracle.nlist_rows(orc["nn"], orc["nm"], n)
    t = case.itype
    for i in range(n):
        keep = rows[i][t[rows[i]] == t[i]]
        got = nn.reshape(-1, nm.shape[0])[:nm[i], i]
        assert np.array_equal(got, keep), i


@pytest.mark.parametrize("pair_tpa,depth", [(8, 2), (4, 0), (16, 1)])
def test_fused_step_matches_separate(pair_tpa, depth):
    """One kernel per leapfrog step (pair forces and update fused) against
    the two-kernel step with the same lanes per atom.  The update performs
    the same FP64 operations, both sum the kinetic energy per (atom, axis)
    term in fixed point and both run the same pair loop, so the runs agree
    bit for bit.  40 steps include list rebuilds."""
    case = oracle.load(_write(synth.nacl_rocksalt(ncell=6, seed=41, nmaxlist=512)))
    out = []
    for fused in (0, 1):
        with gu.system_from_case(case) as sim:
            sim.set_tuning(pair_tpa, 0, depth)
            sim.set_fused_step(fused)
            sim.step(40)
            out.append((sim.positions(), sim.velocities(), sim.thermo(), sim.info()))
    (x0, v0, t0, i0), (x1, v1, t1, i1) = out
    assert i0["kernels_per_step"] == 2 and i1["kernels_per_step"] == 1
    assert i0["builds"] == i1["builds"] >= 2
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1)
    assert t0["ke"] == t1["ke"] and t0["lambda_"] == t1["lambda_"]


@pytest.mark.parametrize("name", ["nacl_fused", "nacl", "argon_vv", "water_nh"])
def test_graph_rebuild_inline_matches_conditional(name):
    """Step graphs with the list-rebuild passes inline (programmatic launches
    that return at once unless a rebuild is due) advance bit for bit like
    graphs with a conditional rebuild node: the same steps rebuild."""
    if name.startswith("nacl"):
        sys_ = synth.nacl_rocksalt(ncell=6, seed=42, nmaxlist=512)
    elif name == "argon_vv":
        sys_ = synth.argon_fcc(ncell=7, seed=3)
    else:
        sys_ = synth.water_grid(nside=9, seed=4)
    case = oracle.load(_write(sys_))
    out = []
    for inline in (0, 1):
        with gu.system_from_case(case) as sim:
            sim.set_tuning(8, 0)
            if name.startswith("nacl"):
                sim.set_fused_step(name == "nacl_fused")
            sim.set_graph_rebuild(inline)
            sim.step(96)
            out.append((sim.positions(), sim.velocities(), sim.info(), sim.thermo()))
    (x0, v0, i0, t0), (x1, v1, i1, t1) = out
    assert i1["kernels_per_rebuild"] == 0 and i0["kernels_per_rebuild"] > 0
    assert i0["builds"] == i1["builds"] >= 2
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1)
    assert t0["ke"] == t1["ke"]


def test_autotune_keeps_results():
    """After autotuning (which may advance the system), list and forces of the
    current positions still match the oracle."""
    case = oracle.load(_write(synth.nacl_rocksalt(ncell=5, seed=40, nmaxlist=512)))
    with gu.system_from_case(case) as sim:
        pt, lt = sim.autotune()
        assert pt in (2, 4, 8, 16) and lt in (0, 4, 8, 16)
        sim.update_neighbors(force=True)
        sim.compute_forces(TERM_PAIR)
        F = sim.forces()
        nn, nm = sim.neighbor_list(512)
        case.pos = np.ascontiguousarray(sim.positions().astype(np.float32))
    orc = gu.oracle_state(case)
    n = case.natom
    assert gu.rms_rel(F[:, :3], orc["f64"][:, :3]) <= FORCE_TOL
    assert np.array_equal(gu.rows_canonical(nn, nm, n, 512), gu.rows_canonical(orc["nn"], orc["nm"], n, 512))


def _drift_kt_per_atom_ns(e, n, dt_fs, t0):
    """Linear-fit slope of the total energy, per atom, in kT per ns."""
    t_ns = np.arange(len(e)) * dt_fs * 1e-6
    slope = np.polyfit(t_ns, e, 1)[0]
    return slope / n / (8.314e-3 * t0)


def test_nve_energy_conservation_argon():
    """Velocity-Verlet NVE of LJ argon (reduced units mapped to A, fs) against
    the FP64 plain form of the same run: the energy trajectories agree while
    the two runs are still close (first 200 steps), and the GPU run conserves
    energy as well as the FP64 plain form does (fluctuation of the total
    energy per atom, in kT, within 1.5x; drift printed for the record)."""
    case = oracle.load(_write(synth.argon_fcc(ncell=5, seed=6, integrator="vv")))
    nsteps = 2000
    x = case.pos.astype(np.float64).copy()
    v = case.vel.astype(np.float64).copy()
    st, rec = oracle.md_plain_run(case, x, v, nsteps, 1)
    with gu.system_from_case(case, integrator=MD_VV) as sim:
        sim.step(nsteps, energy_every=1)
        hist = sim.history(nsteps)
    n = case.natom
    kt = 8.314e-3 * 0.72 / 8.314e-3
    e_gpu = np.array([h["ke"] + h["pe"] for h in hist])
    e_ref = rec[:, 0] + rec[:, 1]
    assert np.abs(e_gpu[:200] - e_ref[:200]).max() / n <= 1e-5 * kt
    fl_gpu = np.std(e_gpu) / n / kt
    fl_ref = np.std(e_ref) / n / kt
    t0 = 0.72 / 8.314e-3
    d_gpu = _drift_kt_per_atom_ns(e_gpu, n, 0.5, t0)
    d_ref = _drift_kt_per_atom_ns(e_ref, n, 0.5, t0)
    print(f"NVE: fluctuation GPU {fl_gpu:.3e} FP64 {fl_ref:.3e} kT/atom; "
          f"drift GPU {d_gpu:.3e} FP64 {d_ref:.3e} kT/atom/ns over 1 ps")
    assert fl_gpu <= 1.5 * fl_ref + 1e-6
