"""Loading of the golden vectors (tests/golden/*.npz) and rebuilding the
cases they were made from.  The goldens were produced by the reference's own
parser and kernels executed on the CPU (tests/golden/make_golden.py)."""
from __future__ import annotations

import hashlib
import json
import os
import tempfile

import numpy as np

import oracle
from md_gpu_gb300 import synth

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF_ROOT = oracle.REF_ROOT


def names():
    with open(os.path.join(GOLDEN_DIR, "index.json")) as fh:
        return list(json.load(fh).keys())


def load_golden(name):
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    g = {k: z[k] for k in z.files}
    g["hashes"] = json.loads(str(g["hashes"]))
    g["meta"] = json.loads(str(g["meta"]))
    return g


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def write_synth(spec, directory):
    spec = dict(spec)
    fn = getattr(synth, spec.pop("fn"))
    return synth.write_case(fn(**spec), directory, "case")


def case_from_golden(g) -> oracle.Case:
    """An oracle.Case for a golden: synthetic cases are regenerated and parsed
    by the oracle; example cases are rebuilt from their stored parsed arrays."""
    meta = g["meta"]
    if meta["kind"] == "synth":
        with tempfile.TemporaryDirectory() as td:
            return oracle.load(write_synth(meta["spec"], td))
    pv = g["params"]
    p = oracle.Params()
    p.rcutsq, p.reacf, p.alfa, p.skin = (float(x) for x in pv[:4])
    p.nmaxlist, p.dt, p.temper_0 = int(pv[4]), float(pv[5]), float(pv[6])
    p.lkspace, p.enstype, p.timrun, p.rdel = int(pv[7]), int(pv[8]), int(pv[9]), float(pv[10])
    p.tau_t = 100.0
    f = oracle.FField()
    cnt = g["fld_counts"]
    f.ntype, f.tbonds, f.tangle = int(cnt[0]), int(cnt[1]), int(cnt[2])
    for k in range(f.ntype):
        f.mass[k] = float(g["mass"][k])
    for k in range(64):
        f.lj1[k] = float(g["lj1"][k]); f.lj2[k] = float(g["lj2"][k])
    for k in range(8):
        f.bnd1[k] = float(g["bnd1"][k]); f.bnd2[k] = float(g["bnd2"][k])
        f.ang1[k] = float(g["ang1"][k]); f.ang2[k] = float(g["ang2"][k])
    n = int(g["itype"].shape[0])
    pos_in = g["pos_in"].reshape(n, 4)
    vel_in = g["vel_in"].reshape(n, 4)
    box = g["box"][:3].astype(np.float32)
    return oracle.Case(params=p, fld=f, natom=n, box=box, boxi=g["box"][3:].astype(np.float32),
                       itype=g["itype"].astype(np.int32), q=pos_in[:, 3].copy(),
                       pos=np.ascontiguousarray(pos_in[:, :3]), vel=np.ascontiguousarray(vel_in[:, :3]),
                       mass=vel_in[:, 3].copy(),
                       bonds=g["bonds"].reshape(-1, 3).astype(np.int32),
                       angles=g["angles"].reshape(-1, 4).astype(np.int32))


def rows_canonical(nn, nm, n, width):
    """Row-major (N, width) neighbour table with 0xffffffff fill, as the golden stores it."""
    pt = nm.shape[0]
    out = np.full((n, width), 0xFFFFFFFF, np.uint32)
    cols = nn.reshape(-1, pt)
    for k in range(width):
        m = nm[:n] > k
        out[m, k] = cols[k, :n][m]
    return out


def case_arrays(case, integrator=None, nmaxlist=None, tau_t=100.0):
    """MDSystem.from_arrays keyword arguments for the inputs the oracle sees."""
    p = case.params
    nt = case.fld.ntype
    bonds = case.bonds.copy()
    angles = case.angles.copy()
    if len(bonds):
        bonds -= 1          # file convention (1-based) -> 0-based
    if len(angles):
        angles -= 1
    tm = np.ctypeslib.as_array(case.fld.mass)[:nt].astype(np.float32)
    lj1 = np.ctypeslib.as_array(case.fld.lj1)[:nt * nt].astype(np.float32)
    lj2 = np.ctypeslib.as_array(case.fld.lj2)[:nt * nt].astype(np.float32)
    arr = lambda k: np.ctypeslib.as_array(getattr(case.fld, k)).astype(np.float32)
    return dict(
        box=case.box, itype=case.itype, charge=case.q, pos=case.pos, vel=case.vel, type_mass=tm,
        lj1=lj1, lj2=lj2, lkspace=p.lkspace, rcutsq=p.rcutsq, reacf=p.reacf, alfa=p.alfa,
        skin=p.skin, nmaxlist=nmaxlist or p.nmaxlist, dt=p.dt, enstype=p.enstype,
        temper_0=p.temper_0, tau_t=tau_t,
        integrator=p.integrator if integrator is None else integrator,
        bonds=bonds if len(bonds) else None, bnd1=arr("bnd1"), bnd2=arr("bnd2"),
        angles=angles if len(angles) else None, ang1=arr("ang1"), ang2=arr("ang2"))


def system_from_case(case, integrator=None, nmaxlist=None, tau_t=100.0, stream=None):
    """The same inputs the oracle sees, uploaded through the C ABI."""
    from md_gpu_gb300 import MDSystem
    return MDSystem.from_arrays(stream=stream, **case_arrays(case, integrator, nmaxlist, tau_t))


def oracle_state(case):
    """Oracle list (reference layout) and FP64 plain-form forces/energies."""
    p = case.params
    pos4 = case.pos4()
    excl = oracle.exclusions(case.natom, case.bonds)
    nn, nm, mx = oracle.nlist(pos4, case.box, case.boxi, oracle.rskinsq(p.skin, p.rcutsq), excl,
                              max(p.nmaxlist, 1024))
    kind = 0 if p.lkspace == 0 else 1
    f64, ep = oracle.pair_f64(kind, pos4, case.itype, case.q, case.box, nn, nm, case.fld.ntype,
                              case.lj1, case.lj2, p.rcutsq, p.reacf if kind == 0 else 0.0, p.alfa)
    return dict(pos4=pos4, excl=excl, nn=nn, nm=nm, mx=mx, kind=kind, f64=f64, ep64=ep)


def rms_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def water_adjoint(nside, seed, rc, nsteps, **loss):
    """A flexible-water system for the adjoint tests: from_batch keyword
    arrays (velocity Verlet NVE) and the oracle's AdjProblem of the same
    inputs (bonds, angles and their parameter tables included)."""
    from md_gpu_gb300 import MD_VV
    with tempfile.TemporaryDirectory() as td:
        case = oracle.load(synth.write_case(synth.water_grid(nside=nside, seed=seed, rc=rc, integrator="vv"),
                                            td, "w"))
    a = case_arrays(case, integrator=MD_VV)
    a["enstype"] = 0
    nt = case.fld.ntype
    f64 = lambda v: np.asarray(v, np.float64)
    prob = oracle.AdjProblem(
        box=f64(a["box"]), itype=a["itype"], q=f64(a["charge"]), mass=f64(a["type_mass"])[a["itype"]],
        lj1=f64(a["lj1"]).reshape(nt, nt), lj2=f64(a["lj2"]).reshape(nt, nt), x0=f64(a["pos"]),
        v0=f64(a["vel"]), rcutsq=a["rcutsq"], alfa=a["alfa"], dt=a["dt"], nsteps=nsteps,
        bonds=a["bonds"], angles=a["angles"], bnd1=f64(a["bnd1"]), bnd2=f64(a["bnd2"]),
        ang1=f64(a["ang1"]), ang2=f64(a["ang2"]), **loss)
    return a, prob
