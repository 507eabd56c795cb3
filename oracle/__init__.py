"""ctypes bindings of the oracle (oracle.c): a CPU restatement of md_gpu's
force-and-integrate path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of bench.py, as the checker.  The product
(md_gpu_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_EMU = os.path.join(HERE, "_ref", "ref_emu")
# Root of the reference project's source tree (the unmodified md_gpu
# checkout): environment variable MD_GPU_REFERENCE, default /root/reference.
# Only the recipes that compile the CPU-emulated reference and the scripts
# that generate golden vectors read it; nothing does at run time on a
# machine without the reference.
REF_ROOT = os.environ.get("MD_GPU_REFERENCE", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src")

_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so (gcc, OpenMP, -ffp-contract=off)."""
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "oracle.c"))):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return LIB_PATH


def build_ref(ref_src: str = REF_SRC) -> Optional[str]:
    """Compile the CPU-emulated reference kernels when the reference tree exists."""
    if not os.path.isdir(ref_src):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_src}"], check=True)
    return REF_EMU


class Params(C.Structure):
    _fields_ = [("enstype", C.c_int), ("temper_0", C.c_float), ("press_0", C.c_float),
                ("timeq", C.c_int), ("timrun", C.c_int), ("timprn", C.c_int),
                ("dt", C.c_float), ("rcutsq", C.c_float), ("lkspace", C.c_int),
                ("reacf", C.c_float), ("alfa", C.c_float), ("kmax", C.c_int),
                ("skin", C.c_float), ("nmaxlist", C.c_int), ("rdel", C.c_float),
                ("tau_t", C.c_float), ("integrator", C.c_int)]


class FField(C.Structure):
    _fields_ = [("ntype", C.c_int), ("nt", C.c_int * 8), ("name", (C.c_char * 16) * 8),
                ("mass", C.c_float * 8), ("charge", C.c_float * 8),
                ("lj1", C.c_float * 64), ("lj2", C.c_float * 64),
                ("tbonds", C.c_int), ("bnd1", C.c_float * 8), ("bnd2", C.c_float * 8),
                ("tangle", C.c_int), ("ang1", C.c_float * 8), ("ang2", C.c_float * 8),
                ("nbonds", C.c_int), ("nangle", C.c_int),
                ("bonds", C.POINTER(C.c_int)), ("angles", C.POINTER(C.c_int))]


class Config(C.Structure):
    _fields_ = [("natom", C.c_int), ("cftyp", C.c_int), ("box", C.c_float * 3),
                ("boxi", C.c_float * 3), ("itype", C.POINTER(C.c_int)),
                ("q", C.POINTER(C.c_float)), ("pos", C.POINTER(C.c_float)),
                ("vel", C.POINTER(C.c_float)), ("mass", C.POINTER(C.c_float))]


F32 = np.float32
U32 = np.uint32


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        L = _lib
        L.orc_count_pairs.restype = C.c_longlong
        for fn in ("orc_rskinsq", "orc_rmaxdif", "orc_decode_q", "orc_ke_sum_ref",
                   "orc_berendsen_scale", "orc_temperature_ref"):
            getattr(L, fn).restype = C.c_float
        L.orc_rskinsq.argtypes = [C.c_float, C.c_float]
        L.orc_rmaxdif.argtypes = [C.c_float]
        L.orc_decode_q.argtypes = [C.c_float]
        L.orc_berendsen_scale.argtypes = [C.c_float] * 4
        L.orc_temperature_ref.argtypes = [C.c_float, C.c_int]
        L.orc_hilbert3.restype = C.c_ulonglong
        L.orc_hilbert3.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_int]
        L.orc_kinetic_f64.restype = C.c_double
    return _lib


@dataclasses.dataclass
class Case:
    """A parsed run (.inp/.fld/.cfg) with arrays copied into numpy."""

    params: Params
    fld: FField
    natom: int
    box: np.ndarray      # float32 (3,)
    boxi: np.ndarray     # float32 (3,)
    itype: np.ndarray    # int32, 0-based
    q: np.ndarray        # float32
    pos: np.ndarray      # float32 (N,3)
    vel: np.ndarray      # float32 (N,3)
    mass: np.ndarray     # float32 (N,) g/mol*1e4
    bonds: np.ndarray    # int32 (nb,3) type,i,j 1-based
    angles: np.ndarray   # int32 (na,4)

    @property
    def lj1(self):
        return np.ctypeslib.as_array(self.fld.lj1).astype(F32)

    @property
    def lj2(self):
        return np.ctypeslib.as_array(self.fld.lj2).astype(F32)

    def pos4(self):
        out = np.empty((self.natom, 4), F32)
        lib().orc_pack_pos4(self.natom, _p(self.pos, C.c_float), _p(self.itype, C.c_int),
                            _p(self.q, C.c_float), _p(out, C.c_float))
        return out

    def vel4(self):
        out = np.empty((self.natom, 4), F32)
        lib().orc_pack_vel4(self.natom, _p(self.vel, C.c_float), _p(self.mass, C.c_float),
                            _p(out, C.c_float))
        return out


def load(base: str) -> Case:
    """Parse <base>.inp/.fld/.cfg with the oracle's restatement of simulation.cu."""
    L = lib()
    p, f, c = Params(), FField(), Config()
    if L.orc_read_inp((base + ".inp").encode(), C.byref(p)):
        raise IOError("bad .inp " + base)
    if L.orc_read_fld((base + ".fld").encode(), C.byref(f)):
        raise IOError("bad .fld " + base)
    if L.orc_read_cfg((base + ".cfg").encode(), C.byref(f), C.byref(c)):
        raise IOError("bad .cfg " + base)
    n = c.natom
    arr = lambda ptr, k, dt: np.ctypeslib.as_array(ptr, shape=(k,)).astype(dt).copy()
    bonds = arr(f.bonds, 3 * f.nbonds, np.int32).reshape(-1, 3) if f.nbonds else np.zeros((0, 3), np.int32)
    angles = arr(f.angles, 4 * f.nangle, np.int32).reshape(-1, 4) if f.nangle else np.zeros((0, 4), np.int32)
    case = Case(params=p, fld=f, natom=n, box=np.array(c.box[:], F32), boxi=np.array(c.boxi[:], F32),
                itype=arr(c.itype, n, np.int32), q=arr(c.q, n, F32),
                pos=arr(c.pos, 3 * n, F32).reshape(n, 3), vel=arr(c.vel, 3 * n, F32).reshape(n, 3),
                mass=arr(c.mass, n, F32), bonds=bonds, angles=angles)
    L.orc_free_cfg(C.byref(c))
    L.orc_free_fld(C.byref(f))
    case.fld.bonds = C.POINTER(C.c_int)()
    case.fld.angles = C.POINTER(C.c_int)()
    return case


def pitch(n):
    return lib().orc_pitch(n)


def rskinsq(skin, rcutsq):
    return F32(lib().orc_rskinsq(skin, rcutsq))


def rmaxdif(skin):
    return F32(lib().orc_rmaxdif(skin))


def wolf_consts(alfa, rcutsq):
    out = np.zeros(4, F32)
    lib().orc_wolf_consts(C.c_float(alfa), C.c_float(rcutsq), _p(out, C.c_float))
    return out


def exclusions(n, bonds):
    ex = np.zeros((n, 4), U32)
    b = np.ascontiguousarray(bonds, np.int32)
    lib().orc_build_exclusions(n, b.shape[0], _p(b, C.c_int), _p(ex, C.c_uint))
    return ex


def nlist(pos4, box, boxi, rsk, excl, nmax):
    """Reference-layout O(N^2) list: (nnlist[pitch*nmax], nnlist_max[pitch], maxcount)."""
    n = pos4.shape[0]
    pt = pitch(n)
    nn = np.zeros(pt * nmax, U32)
    nm = np.zeros(pt, U32)
    mx = lib().orc_nlist_nsquared(n, _p(pos4, C.c_float), _p(box, C.c_float), _p(boxi, C.c_float),
                                  C.c_float(rsk), _p(excl, C.c_uint), pt, nmax,
                                  _p(nn, C.c_uint), _p(nm, C.c_uint))
    return nn, nm, mx


def nlist_rows(nn, nm, n):
    """Per-atom sorted neighbour arrays from the column-major layout."""
    pt = nm.shape[0]
    mx = int(nm[:n].max()) if n else 0
    cols = nn.reshape(-1, pt)[:mx, :n].T
    return [cols[i, :nm[i]] for i in range(n)]


def nlist_check(pos4, pos_old4, box, boxi, rmd):
    n = pos4.shape[0]
    return lib().orc_nlist_check(n, _p(pos4, C.c_float), _p(pos_old4, C.c_float), _p(box, C.c_float),
                                 _p(boxi, C.c_float), C.c_float(rmd))


def pair_f32(kind, pos4, box, boxi, nn, nm, ntype, lj1, lj2, rcutsq, reacf, wc):
    n = pos4.shape[0]
    out = np.zeros((n, 4), F32)
    lib().orc_pair_f32(kind, n, _p(pos4, C.c_float), _p(box, C.c_float), _p(boxi, C.c_float),
                       _p(nn, C.c_uint), _p(nm, C.c_uint), nm.shape[0], ntype,
                       _p(lj1, C.c_float), _p(lj2, C.c_float), C.c_float(rcutsq), C.c_float(reacf),
                       _p(wc, C.c_float), _p(out, C.c_float))
    return out


def pair_f64(kind, pos4, itype, q, box, nn, nm, ntype, lj1, lj2, rcutsq, reacf, alfa,
             erfc_exact=0):
    n = pos4.shape[0]
    out = np.zeros((n, 4), np.float64)
    ep = np.zeros(n, np.float64)
    it = np.ascontiguousarray(itype, np.int32)
    qq = np.ascontiguousarray(q, F32)
    lib().orc_pair_f64(kind, erfc_exact, n, _p(pos4, C.c_float), _p(it, C.c_int), _p(qq, C.c_float),
                       _p(box, C.c_float), _p(nn, C.c_uint), _p(nm, C.c_uint), nm.shape[0], ntype,
                       _p(lj1, C.c_float), _p(lj2, C.c_float), C.c_float(rcutsq), C.c_float(reacf),
                       C.c_float(alfa), _p(out, C.c_double), _p(ep, C.c_double))
    return out, ep


def count_pairs(pos4, box, rcutsq, excl=None):
    n = pos4.shape[0]
    ex = _p(excl, C.c_uint) if excl is not None else None
    return lib().orc_count_pairs(n, _p(pos4, C.c_float), _p(box, C.c_float), C.c_float(rcutsq), ex)


def bond_lists(n, bonds, pt):
    bl = np.zeros((4 * pt, 2), U32)
    bm = np.zeros(pt, U32)
    b = np.ascontiguousarray(bonds, np.int32)
    if lib().orc_bond_lists(n, b.shape[0], _p(b, C.c_int), pt, _p(bl, C.c_uint), _p(bm, C.c_uint)):
        raise ValueError("more than four bonds on an atom")
    return bl, bm


def angle_lists(n, angles, pt):
    al = np.zeros((4 * pt, 4), U32)
    am = np.zeros(pt, U32)
    a = np.ascontiguousarray(angles, np.int32)
    if lib().orc_angle_lists(n, a.shape[0], _p(a, C.c_int), pt, _p(al, C.c_uint), _p(am, C.c_uint)):
        raise ValueError("more than four angles on an atom")
    return al, am


def bonds_f32(pos4, box, boxi, bl, bm, bnd1, bnd2, force4):
    n = pos4.shape[0]
    lib().orc_bonds_f32(n, _p(pos4, C.c_float), _p(box, C.c_float), _p(boxi, C.c_float),
                        _p(bl, C.c_uint), _p(bm, C.c_uint), bm.shape[0], _p(bnd1, C.c_float),
                        _p(bnd2, C.c_float), _p(force4, C.c_float))


def angles_f32(pos4, box, boxi, al, am, ang1, ang2, force4):
    n = pos4.shape[0]
    lib().orc_angles_f32(n, _p(pos4, C.c_float), _p(box, C.c_float), _p(boxi, C.c_float),
                         _p(al, C.c_uint), _p(am, C.c_uint), am.shape[0], _p(ang1, C.c_float),
                         _p(ang2, C.c_float), _p(force4, C.c_float))


def bonds_f64(pos4, box, bonds, bnd1, bnd2, force4, epot):
    b = np.ascontiguousarray(bonds, np.int32)
    lib().orc_bonds_f64(pos4.shape[0], _p(pos4, C.c_float), _p(box, C.c_float), b.shape[0],
                        _p(b, C.c_int), _p(bnd1, C.c_float), _p(bnd2, C.c_float),
                        _p(force4, C.c_double), _p(epot, C.c_double))


def angles_f64(pos4, box, angles, ang1, ang2, force4, epot):
    a = np.ascontiguousarray(angles, np.int32)
    lib().orc_angles_f64(pos4.shape[0], _p(pos4, C.c_float), _p(box, C.c_float), a.shape[0],
                         _p(a, C.c_int), _p(ang1, C.c_float), _p(ang2, C.c_float),
                         _p(force4, C.c_double), _p(epot, C.c_double))


def leapfrog_nve_f32(pos4, vel4, force4, dt, box, boxi):
    n = pos4.shape[0]
    lib().orc_leapfrog_nve_f32(n, _p(pos4, C.c_float), _p(vel4, C.c_float), _p(force4, C.c_float),
                               C.c_float(dt), _p(box, C.c_float), _p(boxi, C.c_float))


def leapfrog_nvt_f32(pos4, vel4, force4, dt, scale, box, boxi, block=256):
    n = pos4.shape[0]
    nb = (n + block - 1) // block
    part = np.zeros(nb, F32)
    lib().orc_leapfrog_nvt_f32(n, _p(pos4, C.c_float), _p(vel4, C.c_float), _p(force4, C.c_float),
                               C.c_float(dt), C.c_float(scale), _p(box, C.c_float),
                               _p(boxi, C.c_float), block, _p(part, C.c_float))
    return part


def ke_sum_ref(part):
    part = np.ascontiguousarray(part, F32)
    return F32(lib().orc_ke_sum_ref(part.shape[0], _p(part, C.c_float)))


def berendsen_scale(dt, tco, t0, t):
    return F32(lib().orc_berendsen_scale(dt, tco, t0, t))


def temperature_ref(ke0, n):
    return F32(lib().orc_temperature_ref(C.c_float(ke0), n))


def vv_pre_f32(pos4, vel4, force4, dt, box, boxi):
    lib().orc_vv_pre_f32(pos4.shape[0], _p(pos4, C.c_float), _p(vel4, C.c_float), _p(force4, C.c_float),
                         C.c_float(dt), _p(box, C.c_float), _p(boxi, C.c_float))


def vv_cor_f32(vel4, force4, dt):
    lib().orc_vv_cor_f32(vel4.shape[0], _p(vel4, C.c_float), _p(force4, C.c_float), C.c_float(dt))


def cell_dims(box, rl):
    nc = np.zeros(3, np.int32)
    bl = np.zeros(3, F32)
    lib().orc_cell_dims(_p(box, C.c_float), C.c_float(rl), _p(nc, C.c_int), _p(bl, C.c_float))
    return nc, bl


def cell_index(pos4, box, nc, bl):
    n = pos4.shape[0]
    out = np.zeros((n, 3), np.int32)
    lib().orc_cell_index(n, _p(pos4, C.c_float), _p(box, C.c_float), _p(nc, C.c_int),
                         _p(bl, C.c_float), _p(out, C.c_int))
    return out


def hilbert3(x, y, z, bits):
    return lib().orc_hilbert3(x, y, z, bits)


def md_ref_run(case: Case, pos4, vel4, nsteps, exact_ke=0, temper=None):
    """The reference step loop in FP32 as written; returns (builds, force4, temps, temper)."""
    n = pos4.shape[0]
    f4 = np.zeros((n, 4), F32)
    temps = np.zeros(max(nsteps, 1), F32)
    t = C.c_float(case.params.temper_0 if temper is None else temper)
    fld = case.fld
    b = np.ascontiguousarray(case.bonds, np.int32)
    a = np.ascontiguousarray(case.angles, np.int32)
    fld.nbonds, fld.nangle = b.shape[0], a.shape[0]
    fld.bonds = _p(b, C.c_int)
    fld.angles = _p(a, C.c_int)
    rc = lib().orc_md_ref_run(C.byref(case.params), C.byref(fld), n, _p(pos4, C.c_float),
                              _p(vel4, C.c_float), _p(case.box, C.c_float), _p(case.boxi, C.c_float),
                              nsteps, exact_ke, _p(f4, C.c_float), C.byref(t), _p(temps, C.c_float))
    fld.bonds = C.POINTER(C.c_int)()
    fld.angles = C.POINTER(C.c_int)()
    return rc, f4, temps[:nsteps], float(t.value)


class RefLoopState:
    """The list the reference's loop keeps between steps (for md_ref_run_cont)."""

    def __init__(self, n, nmaxlist):
        pitch = ((n + 255) // 256) * 256
        self.nnl = np.zeros(pitch * nmaxlist, np.uint32)
        self.nnm = np.zeros(pitch, np.uint32)
        self.pold = np.zeros((n, 4), F32)
        self.have = C.c_int(0)


def md_ref_run_cont(case: Case, pos4, vel4, nsteps, state: RefLoopState, temper=None):
    """md_ref_run continuing from the list in `state` (built on the first call):
    the reference's loop over consecutive calls, rebuilding only on its
    displacement criterion; returns (builds in this call, temper)."""
    n = pos4.shape[0]
    t = C.c_float(case.params.temper_0 if temper is None else temper)
    fld = case.fld
    b = np.ascontiguousarray(case.bonds, np.int32)
    a = np.ascontiguousarray(case.angles, np.int32)
    fld.nbonds, fld.nangle = b.shape[0], a.shape[0]
    fld.bonds = _p(b, C.c_int)
    fld.angles = _p(a, C.c_int)
    rc = lib().orc_md_ref_run_cont(C.byref(case.params), C.byref(fld), n, _p(pos4, C.c_float),
                                   _p(vel4, C.c_float), _p(case.box, C.c_float), _p(case.boxi, C.c_float),
                                   nsteps, 0, _p(state.nnl, C.c_uint), _p(state.nnm, C.c_uint),
                                   _p(state.pold, C.c_float), C.byref(state.have), None, C.byref(t), None)
    fld.bonds = C.POINTER(C.c_int)()
    fld.angles = C.POINTER(C.c_int)()
    return rc, float(t.value)


BAR = 16605.3907   # bar per kJ/mol/A^3


def md_plain_npt(case: Case, x, v, nsteps, press_bar, tau_p_fs, beta_per_bar, mu_max=1e-4):
    """FP64 plain-form NPT run (Berendsen leapfrog thermostat and barostat,
    all pairs, small N); x, v (N, 3) float64 in/out.  Returns (box[3],
    records[nsteps, 4] = Lx, P (bar), T, the scale the step applied)."""
    n = x.shape[0]
    m = case.mass.astype(np.float64)
    box = case.box.astype(np.float64).copy()
    rec = np.zeros((max(nsteps, 1), 4))
    fld = case.fld
    b = np.ascontiguousarray(case.bonds, np.int32)
    a = np.ascontiguousarray(case.angles, np.int32)
    fld.nbonds, fld.nangle = b.shape[0], a.shape[0]
    fld.bonds = _p(b, C.c_int)
    fld.angles = _p(a, C.c_int)
    it = np.ascontiguousarray(case.itype, np.int32)
    mu_k = beta_per_bar * BAR * float(case.params.dt) / (3.0 * tau_p_fs)
    L = lib()
    L.orc_md_plain_npt.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double,
                                   C.c_double, C.c_void_p]
    rc = L.orc_md_plain_npt(C.addressof(case.params), C.addressof(fld), n, x.ctypes.data, v.ctypes.data,
                            it.ctypes.data, case.q.ctypes.data, m.ctypes.data, box.ctypes.data, nsteps,
                            press_bar / BAR, mu_k, mu_max, rec.ctypes.data)
    fld.bonds = C.POINTER(C.c_int)()
    fld.angles = C.POINTER(C.c_int)()
    if rc != 0:
        raise ValueError("orc_md_plain_npt: angles are not supported")
    rec[:, 1] *= BAR
    return box, rec[:nsteps]


def md_plain_run(case: Case, x, v, nsteps, integrator, state=None, records=True):
    """FP64 plain-form run (all pairs, small N); returns (state[4], records[nsteps,3])."""
    n = x.shape[0]
    m = case.mass.astype(np.float64)
    st = np.zeros(4) if state is None else np.array(state, np.float64)
    rec = np.zeros((max(nsteps, 1), 3)) if records else None
    fld = case.fld
    b = np.ascontiguousarray(case.bonds, np.int32)
    a = np.ascontiguousarray(case.angles, np.int32)
    fld.nbonds, fld.nangle = b.shape[0], a.shape[0]
    fld.bonds = _p(b, C.c_int)
    fld.angles = _p(a, C.c_int)
    it = np.ascontiguousarray(case.itype, np.int32)
    lib().orc_md_plain_run(C.byref(case.params), C.byref(fld), n, _p(x, C.c_double), _p(v, C.c_double),
                           _p(it, C.c_int), _p(case.q, C.c_float), _p(m, C.c_double),
                           _p(case.box, C.c_float), nsteps, integrator, _p(st, C.c_double),
                           _p(rec, C.c_double) if rec is not None else None)
    fld.bonds = C.POINTER(C.c_int)()
    fld.angles = C.POINTER(C.c_int)()
    return st, (rec[:nsteps] if rec is not None else None)


# ---- adjoint of velocity-Verlet NVE (FP64, all pairs; small N) ----

class AdjCfg(C.Structure):
    _fields_ = [("natom", C.c_int), ("ntype", C.c_int), ("nsteps", C.c_int),
                ("box", C.c_double * 3), ("rcutsq", C.c_double), ("alfa", C.c_double),
                ("dt", C.c_double), ("w_pe", C.c_double), ("w_rdf", C.c_double),
                ("rdf_a", C.c_int), ("rdf_b", C.c_int), ("nbins", C.c_int),
                ("rdf_dr", C.c_double), ("rdf_sigma", C.c_double),
                ("nbonds", C.c_int), ("nangles", C.c_int), ("bonds", C.c_void_p), ("angles", C.c_void_p),
                ("bnd1", C.c_void_p), ("bnd2", C.c_void_p), ("ang1", C.c_void_p), ("ang2", C.c_void_p)]


@dataclasses.dataclass
class AdjProblem:
    """One system and loss for the FP64 adjoint: arrays in FP64, masses per
    atom in g/mol*1e4, LJ tables ntype x ntype, charges q (scale 1)."""

    box: np.ndarray
    itype: np.ndarray
    q: np.ndarray
    mass: np.ndarray
    lj1: np.ndarray
    lj2: np.ndarray
    x0: np.ndarray
    v0: np.ndarray
    rcutsq: float
    alfa: float
    dt: float
    nsteps: int
    w_pe: float = 1.0
    w_rdf: float = 1.0
    rdf_a: int = 0
    rdf_b: int = 1
    nbins: int = 200
    rdf_dr: float = 0.05
    rdf_sigma: float = 0.05
    bonds: Optional[np.ndarray] = None    # (nb, 3): type, i, j (0-based)
    angles: Optional[np.ndarray] = None   # (na, 4): type, i, j (centre), k
    bnd1: Optional[np.ndarray] = None     # per type, 2k
    bnd2: Optional[np.ndarray] = None     # per type, r0
    ang1: Optional[np.ndarray] = None     # per type, 2k
    ang2: Optional[np.ndarray] = None     # per type, theta0 (rad)

    def cfg(self):
        c = AdjCfg()
        c.natom, c.ntype, c.nsteps = len(self.itype), int(np.asarray(self.lj1).shape[0]), self.nsteps
        for k in range(3):
            c.box[k] = float(self.box[k])
        c.rcutsq, c.alfa, c.dt = self.rcutsq, self.alfa, self.dt
        c.w_pe, c.w_rdf = self.w_pe, self.w_rdf
        c.rdf_a, c.rdf_b, c.nbins = self.rdf_a, self.rdf_b, self.nbins
        c.rdf_dr, c.rdf_sigma = self.rdf_dr, self.rdf_sigma
        # the arrays stay alive with the cfg (it holds their addresses)
        c._keep = []

        def arr(a, t):
            a = np.ascontiguousarray(a, t)
            c._keep.append(a)
            return a.ctypes.data

        zero8 = np.zeros(8)
        if self.bonds is not None and len(self.bonds):
            c.nbonds = len(self.bonds)
            c.bonds = arr(np.asarray(self.bonds).reshape(-1), np.int32)
        if self.angles is not None and len(self.angles):
            c.nangles = len(self.angles)
            c.angles = arr(np.asarray(self.angles).reshape(-1), np.int32)
        for k in ("bnd1", "bnd2", "ang1", "ang2"):
            v = getattr(self, k)
            setattr(c, k, arr(zero8 if v is None else v, np.float64))
        return c

    def _arrays(self, lj1=None, lj2=None, q=None):
        d = lambda a: np.ascontiguousarray(a, np.float64)
        return (np.ascontiguousarray(self.itype, np.int32), d(self.q if q is None else q), d(self.mass),
                d(self.lj1 if lj1 is None else lj1).reshape(-1), d(self.lj2 if lj2 is None else lj2).reshape(-1),
                d(self.x0).reshape(-1), d(self.v0).reshape(-1))


def adj_loss(prob: AdjProblem, target=None, lj1=None, lj2=None, q=None):
    """Loss of the FP64 forward run; returns (loss, gbar, mean PE)."""
    L = lib()
    L.orc_adj_loss.restype = C.c_double
    c = prob.cfg()
    it, qq, m, l1, l2, x0, v0 = prob._arrays(lj1, lj2, q)
    tg = None if target is None else np.ascontiguousarray(target, np.float64)
    g = np.zeros(prob.nbins)
    pe = C.c_double()
    loss = L.orc_adj_loss(C.byref(c), _p(it, C.c_int), _p(qq, C.c_double), _p(m, C.c_double),
                          _p(l1, C.c_double), _p(l2, C.c_double), _p(x0, C.c_double), _p(v0, C.c_double),
                          _p(tg, C.c_double) if tg is not None else None, _p(g, C.c_double), C.byref(pe))
    return loss, g, pe.value


def adj_grad(prob: AdjProblem, target=None):
    """Loss and its FP64 adjoint gradient: (loss, dlj1[nt,nt], dlj2[nt,nt], dlns, gbar)."""
    L = lib()
    L.orc_adj_grad.restype = C.c_double
    c = prob.cfg()
    it, qq, m, l1, l2, x0, v0 = prob._arrays()
    nt = c.ntype
    tg = None if target is None else np.ascontiguousarray(target, np.float64)
    d1, d2, g = np.zeros(nt * nt), np.zeros(nt * nt), np.zeros(prob.nbins)
    ds = C.c_double()
    loss = L.orc_adj_grad(C.byref(c), _p(it, C.c_int), _p(qq, C.c_double), _p(m, C.c_double),
                          _p(l1, C.c_double), _p(l2, C.c_double), _p(x0, C.c_double), _p(v0, C.c_double),
                          _p(tg, C.c_double) if tg is not None else None, _p(d1, C.c_double),
                          _p(d2, C.c_double), C.byref(ds), _p(g, C.c_double))
    return loss, d1.reshape(nt, nt), d2.reshape(nt, nt), ds.value, g
