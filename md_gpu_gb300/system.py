"""Python mirror of the C ABI (include/md_gpu.h) over ctypes.

This is the host-side interface a user of md_gpu's step loop calls: create a
system from the reference's .inp/.fld/.cfg files or from arrays, step it,
read positions, velocities, forces, energies, neighbour lists and the per
step thermodynamic records.  All compute happens in libmdgpu_gb300.so; there
is no CPU path, and loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmdgpu_gb300.so")

MD_LEAPFROG, MD_VV, MD_NH = 0, 1, 2
TERM_PAIR, TERM_BOND, TERM_ANGLE, TERM_RECIP, TERM_ALL = 1, 2, 4, 8, 15
STATUS = {0: "ok", 1: "invalid argument", 2: "cannot open file", 3: "parse error", 4: "CUDA error",
          5: "neighbour list overflow", 6: "more than four bonds/angles on an atom",
          7: "unsupported option", 8: "cutoff + skin exceeds half the box"}


class MDError(RuntimeError):
    def __init__(self, status, msg=""):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class SystemDesc(C.Structure):
    _fields_ = [("natom", C.c_int), ("ntype", C.c_int), ("box", C.c_float * 3),
                ("itype", C.POINTER(C.c_int)), ("charge", C.POINTER(C.c_float)),
                ("pos", C.POINTER(C.c_float)), ("vel", C.POINTER(C.c_float)),
                ("type_mass", C.POINTER(C.c_float)), ("lj1", C.POINTER(C.c_float)),
                ("lj2", C.POINTER(C.c_float)), ("nbonds", C.c_int), ("bonds", C.POINTER(C.c_int)),
                ("bnd1", C.POINTER(C.c_float)), ("bnd2", C.POINTER(C.c_float)),
                ("nangle", C.c_int), ("angles", C.POINTER(C.c_int)),
                ("ang1", C.POINTER(C.c_float)), ("ang2", C.POINTER(C.c_float)),
                ("lkspace", C.c_int), ("rcutsq", C.c_float), ("reacf", C.c_float),
                ("alfa", C.c_float), ("skin", C.c_float), ("nmaxlist", C.c_int),
                ("enstype", C.c_int), ("temper_0", C.c_float), ("dt", C.c_float),
                ("tau_t", C.c_float), ("integrator", C.c_int)]


class Thermo(C.Structure):
    _fields_ = [("step", C.c_longlong), ("ke", C.c_double), ("temper", C.c_double),
                ("pe", C.c_double), ("virial", C.c_double), ("conserved", C.c_double),
                ("xi", C.c_double), ("lambda_", C.c_double), ("builds", C.c_int),
                ("flags", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdjointCfg(C.Structure):
    _fields_ = [("nsteps", C.c_int), ("checkpoint", C.c_int), ("gradient", C.c_int),
                ("w_pe", C.c_double), ("w_rdf", C.c_double), ("rdf_a", C.c_int), ("rdf_b", C.c_int),
                ("nbins", C.c_int), ("rdf_dr", C.c_double), ("rdf_sigma", C.c_double)]


class Info(C.Structure):
    _fields_ = [("natom", C.c_int), ("pitch", C.c_int), ("capacity", C.c_int),
                ("ncell", C.c_int * 3), ("stencil", C.c_int * 3), ("binlen", C.c_float * 3),
                ("pair_threads_per_atom", C.c_int), ("list_threads_per_atom", C.c_int),
                ("builds", C.c_int), ("max_neighbors", C.c_int), ("kernels_per_step", C.c_int),
                ("kernels_per_rebuild", C.c_int), ("kernels_per_graph", C.c_int),
                ("pair_entries_per_lane", C.c_int), ("positions_centered", C.c_int),
                ("fused_step", C.c_int), ("rebuild_inline", C.c_int), ("list_regrows", C.c_int),
                ("cell_regrids", C.c_int), ("pme_grid", C.c_int * 3)]


def _make_desc(keep, *, box, itype, charge, pos, vel, type_mass, lj1, lj2, lkspace, rcutsq,
               skin, nmaxlist, dt, reacf=0.0, alfa=0.0, enstype=0, temper_0=0.0, tau_t=100.0,
               integrator=MD_LEAPFROG, bonds=None, bnd1=None, bnd2=None, angles=None,
               ang1=None, ang2=None) -> SystemDesc:
    """An md_system_desc over numpy copies of the arrays (kept alive in `keep`)."""

    def f32(a):
        a = np.ascontiguousarray(a, np.float32)
        keep.append(a)
        return _ptr(a, C.c_float)

    def i32(a):
        a = np.ascontiguousarray(a, np.int32)
        keep.append(a)
        return _ptr(a, C.c_int)

    n = int(np.asarray(itype).shape[0])
    ntype = int(np.asarray(type_mass).shape[0])
    d = SystemDesc()
    d.natom, d.ntype = n, ntype
    for k in range(3):
        d.box[k] = float(box[k])
    d.itype, d.charge = i32(itype), f32(charge)
    d.pos = f32(np.asarray(pos).reshape(-1))
    d.vel = f32(np.asarray(vel).reshape(-1)) if vel is not None else None
    d.type_mass = f32(type_mass)
    d.lj1, d.lj2 = f32(np.asarray(lj1).reshape(-1)), f32(np.asarray(lj2).reshape(-1))
    pad8 = lambda a: np.pad(np.asarray(a, np.float32), (0, 8 - len(a)))
    if bonds is not None and len(bonds):
        d.nbonds = len(bonds)
        d.bonds = i32(np.asarray(bonds).reshape(-1))
        d.bnd1, d.bnd2 = f32(pad8(bnd1)), f32(pad8(bnd2))
    if angles is not None and len(angles):
        d.nangle = len(angles)
        d.angles = i32(np.asarray(angles).reshape(-1))
        d.ang1, d.ang2 = f32(pad8(ang1)), f32(pad8(ang2))
    d.lkspace, d.rcutsq, d.reacf, d.alfa = lkspace, rcutsq, reacf, alfa
    d.skin, d.nmaxlist, d.enstype, d.temper_0 = skin, nmaxlist, enstype, temper_0
    d.dt, d.tau_t, d.integrator = dt, tau_t, integrator
    return d


_lib = None


def library(path: Optional[str] = None):
    """Load libmdgpu_gb300.so (build it with md_gpu_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libmdgpu_gb300.so not built ({p}); run md_gpu_gb300.build.build()")
    L = C.CDLL(p)
    vp = C.c_void_p
    L.md_status_string.restype = C.c_char_p
    L.md_create.argtypes = [C.POINTER(SystemDesc), vp, C.POINTER(vp)]
    L.md_create_from_files.argtypes = [C.c_char_p, vp, C.POINTER(vp)]
    L.md_destroy.argtypes = [vp]
    for fn in ("md_set_positions", "md_set_velocities", "md_get_positions", "md_get_velocities",
               "md_get_forces", "md_get_energies"):
        getattr(L, fn).argtypes = [vp, vp]
    L.md_update_neighbors.argtypes = [vp, C.c_int]
    L.md_get_neighbor_list.argtypes = [vp, vp, vp, C.c_int, C.c_int]
    L.md_compute_forces.argtypes = [vp, C.c_int, C.c_int]
    L.md_step.argtypes = [vp, C.c_int, C.c_int]
    L.md_get_thermo.argtypes = [vp, C.POINTER(Thermo)]
    L.md_get_thermo_history.argtypes = [vp, C.POINTER(Thermo), C.c_int, C.POINTER(C.c_int)]
    L.md_run_host.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.POINTER(Thermo)]
    L.md_write_cfg.argtypes = [vp, C.c_char_p]
    L.md_write_xyz.argtypes = [vp, C.c_char_p, C.c_int]
    L.md_write_restart.argtypes = [vp, C.c_char_p]
    L.md_read_restart.argtypes = [vp, C.c_char_p]
    L.md_get_info.argtypes = [vp, C.POINTER(Info)]
    L.md_get_order.argtypes = [vp, vp]
    L.md_get_cell_ranks.argtypes = [vp, vp]
    L.md_set_tuning.argtypes = [vp, C.c_int, C.c_int]
    L.md_set_pair_depth.argtypes = [vp, C.c_int]
    L.md_last_step_ms.argtypes = [vp, C.POINTER(C.c_float)]
    L.md_last_error.argtypes = [vp, C.c_char_p, C.c_int]
    L.md_time_pair.argtypes = [vp, C.c_int, C.POINTER(C.c_float)]
    L.md_probe_fp32_peak.argtypes = [C.POINTER(C.c_double)]
    L.md_time_rebuild.argtypes = [vp, C.c_int, C.POINTER(C.c_float)]
    L.md_autotune.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.md_set_type_exclusions.argtypes = [vp, vp]
    L.md_set_graphs.argtypes = [vp, C.c_int]
    L.md_debug_rebuild_barrier.argtypes = [vp, C.c_double, C.c_int]
    L.md_set_precision.argtypes = [vp, C.c_int]
    L.md_set_barostat.argtypes = [vp, C.c_double, C.c_double, C.c_double]
    L.md_set_pme.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    L.md_get_replica_box.argtypes = [vp, vp, vp, C.c_int]
    L.md_debug_list_capacity.argtypes = [vp, C.c_int, C.c_int]
    L.md_get_replica_history.argtypes = [vp, vp, C.c_int, C.POINTER(C.c_int)]
    L.md_set_fused_step.argtypes = [vp, C.c_int]
    L.md_set_graph_rebuild.argtypes = [vp, C.c_int]
    L.md_ref_kinetic_energy_noalloc.argtypes = [vp, C.c_int, vp, vp]
    L.md_create_batch.argtypes = [C.POINTER(SystemDesc), C.c_int, vp, C.POINTER(vp)]
    L.md_get_replica_thermo.argtypes = [vp, C.POINTER(Thermo), C.c_int]
    L.md_adjoint_run.argtypes = [vp, C.POINTER(AdjointCfg), vp, vp, vp, vp, vp, vp]
    _lib = L
    return L


def fp32_peak_tflops():
    """Measured FP32 FMA throughput of the current GPU, TFLOP/s."""
    t = C.c_double()
    _check(library().md_probe_fp32_peak(C.byref(t)))
    return t.value


def _err(ctx=None):
    buf = C.create_string_buffer(1024)
    library().md_last_error(ctx, buf, 1024)
    return buf.value.decode(errors="replace")


def _check(status, ctx=None):
    if status != 0:
        raise MDError(status, _err(ctx))


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class MDSystem:
    """One system resident on the GPU (an md_ctx)."""

    def __init__(self, ctx, natom):
        self._ctx = ctx
        self.natom = natom

    # ---- construction ----
    @classmethod
    def from_files(cls, base: str, stream=None) -> "MDSystem":
        L = library()
        ctx = C.c_void_p()
        _check(L.md_create_from_files(base.encode(), stream, C.byref(ctx)))
        n = Info()
        _check(L.md_get_info(ctx, C.byref(n)), ctx)
        return cls(ctx, n.natom)

    @classmethod
    def from_arrays(cls, *, box, itype, charge, pos, vel, type_mass, lj1, lj2, lkspace, rcutsq,
                    skin, nmaxlist, dt, reacf=0.0, alfa=0.0, enstype=0, temper_0=0.0, tau_t=100.0,
                    integrator=MD_LEAPFROG, bonds=None, bnd1=None, bnd2=None, angles=None,
                    ang1=None, ang2=None, stream=None) -> "MDSystem":
        """Arrays in the reference's in-memory conventions: itype 0-based,
        masses g/mol*1e4 per type, lj tables ntype x ntype, bonds (type,i,j)
        and angles (type,i,j,k) 0-based, bnd1/ang1 = 2k, ang2 in rad."""
        keep = []
        d = _make_desc(keep, box=box, itype=itype, charge=charge, pos=pos, vel=vel,
                       type_mass=type_mass, lj1=lj1, lj2=lj2, lkspace=lkspace, rcutsq=rcutsq,
                       skin=skin, nmaxlist=nmaxlist, dt=dt, reacf=reacf, alfa=alfa,
                       enstype=enstype, temper_0=temper_0, tau_t=tau_t, integrator=integrator,
                       bonds=bonds, bnd1=bnd1, bnd2=bnd2, angles=angles, ang1=ang1, ang2=ang2)
        ctx = C.c_void_p()
        _check(library().md_create(C.byref(d), stream, C.byref(ctx)))
        return cls(ctx, d.natom)

    @classmethod
    def from_batch(cls, replicas, stream=None) -> "MDSystem":
        """A batch of independent replicas (md_create_batch): `replicas` is a
        list of from_arrays keyword dicts.  Positions, velocities, forces and
        energies of the result hold the replicas' atoms concatenated in
        order (see replica_slices); thermo() gives batch totals and
        replica_thermo() the per-replica values."""
        keep = []
        descs = (SystemDesc * len(replicas))()
        sizes = []
        for k, kw in enumerate(replicas):
            descs[k] = _make_desc(keep, **kw)
            sizes.append(descs[k].natom)
        ctx = C.c_void_p()
        _check(library().md_create_batch(descs, len(replicas), stream, C.byref(ctx)))
        sim = cls(ctx, int(sum(sizes)))
        sim.replica_sizes = sizes
        return sim

    def replica_slices(self):
        """Atom ranges of the replicas in the concatenated host arrays."""
        sizes = getattr(self, "replica_sizes", [self.natom])
        off = np.concatenate([[0], np.cumsum(sizes)])
        return [slice(int(off[k]), int(off[k + 1])) for k in range(len(sizes))]

    def replica_thermo(self):
        """Per-replica thermodynamic state after the last step."""
        n = len(getattr(self, "replica_sizes", [self.natom]))
        buf = (Thermo * n)()
        _check(library().md_get_replica_thermo(self._ctx, buf, n), self._ctx)
        return [buf[i].as_dict() for i in range(n)]

    def replica_history(self, n):
        """Per-replica (KE, PE, conserved) of the last min(n, steps, 4096)
        steps of a batch, oldest first: an array (steps, nrep, 3); PE and
        the conserved quantity are 0 on steps without energies.  Returns
        (array, steps) where steps are the step numbers of the rows."""
        nrep = len(getattr(self, "replica_sizes", [self.natom]))
        buf = np.zeros((max(n, 1), nrep, 3))
        got = C.c_int()
        _check(library().md_get_replica_history(self._ctx, buf.ctypes.data, int(n), C.byref(got)), self._ctx)
        k = got.value
        last = self.thermo()["step"]
        return buf[:k], np.arange(last - k + 1, last + 1)

    def adjoint(self, nsteps, checkpoint=50, w_pe=1.0, w_rdf=1.0, rdf_types=(0, 1), nbins=200,
                dr=0.05, sigma=0.05, target=None, gradient=True):
        """Loss of the next `nsteps` velocity-Verlet steps of a batch and its
        adjoint gradient (md_adjoint_run).  Returns a dict with per-replica
        'loss' (nrep,), 'gbar' (nrep, nbins) and, with gradient, 'dlj1',
        'dlj2' (nrep, 8, 8; entry [a, b] as used by atoms of type a) and
        'dlns' (nrep,).  The system advances by nsteps steps."""
        nrep = len(getattr(self, "replica_sizes", [self.natom]))
        cfg = AdjointCfg(nsteps=int(nsteps), checkpoint=int(checkpoint), gradient=1 if gradient else 0,
                         w_pe=float(w_pe), w_rdf=float(w_rdf), rdf_a=int(rdf_types[0]),
                         rdf_b=int(rdf_types[1]), nbins=int(nbins), rdf_dr=float(dr),
                         rdf_sigma=float(sigma))
        loss = np.zeros(nrep)
        gbar = np.zeros((nrep, nbins))
        d1 = np.zeros((nrep, 8, 8))
        d2 = np.zeros((nrep, 8, 8))
        ds = np.zeros(nrep)
        tg = None
        if target is not None:
            tg = np.ascontiguousarray(np.broadcast_to(np.asarray(target, np.float64), (nrep, nbins)))
        _check(library().md_adjoint_run(self._ctx, C.byref(cfg), tg.ctypes.data if tg is not None else None,
                                        loss.ctypes.data, gbar.ctypes.data, d1.ctypes.data,
                                        d2.ctypes.data, ds.ctypes.data), self._ctx)
        out = {"loss": loss, "gbar": gbar}
        if gradient:
            out.update(dlj1=d1, dlj2=d2, dlns=ds)
        return out

    def close(self):
        if self._ctx:
            library().md_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- state ----
    def _get(self, fn, cols):
        out = np.zeros((self.natom, cols), np.float64) if cols > 1 else np.zeros(self.natom)
        _check(getattr(library(), fn)(self._ctx, out.ctypes.data), self._ctx)
        return out

    def positions(self):
        return self._get("md_get_positions", 3)

    def velocities(self):
        return self._get("md_get_velocities", 3)

    def forces(self):
        """(N, 4): fx, fy, fz, sum ff r^2 (kJ/mol/A; kJ/mol)."""
        return self._get("md_get_forces", 4)

    def energies(self):
        return self._get("md_get_energies", 1)

    def set_positions(self, pos):
        a = np.ascontiguousarray(pos, np.float64)
        _check(library().md_set_positions(self._ctx, a.ctypes.data), self._ctx)

    def set_velocities(self, vel):
        a = np.ascontiguousarray(vel, np.float64)
        _check(library().md_set_velocities(self._ctx, a.ctypes.data), self._ctx)

    # ---- work ----
    def update_neighbors(self, force=True):
        _check(library().md_update_neighbors(self._ctx, 1 if force else 0), self._ctx)

    def compute_forces(self, terms=TERM_ALL, energy=False):
        _check(library().md_compute_forces(self._ctx, terms, 1 if energy else 0), self._ctx)

    def step(self, nsteps, energy_every=0):
        _check(library().md_step(self._ctx, int(nsteps), int(energy_every)), self._ctx)

    def last_step_ms(self):
        ms = C.c_float()
        _check(library().md_last_step_ms(self._ctx, C.byref(ms)), self._ctx)
        return ms.value

    def run_host(self, pos, vel, nsteps, energy_every=0, inplace=False, raw_records=False):
        """End to end from host buffers; returns (pos, vel, records).

        inplace: pos and vel (float64, C-contiguous, (N, 3)) are read and
        overwritten by the call itself (pinned buffers then go to the device
        without a staging copy).  raw_records: the records as a NumPy
        structured array over the returned buffer instead of dicts."""
        if inplace:
            for a in (pos, vel):
                if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous
                        and a.size == 3 * self.natom):
                    raise ValueError("inplace run_host needs C-contiguous float64 arrays of N x 3")
            p, v = pos, vel
        else:
            p = np.ascontiguousarray(pos, np.float64).copy()
            v = np.ascontiguousarray(vel, np.float64).copy()
        rec = (Thermo * max(nsteps, 1))()
        _check(library().md_run_host(self._ctx, p.ctypes.data, v.ctypes.data, nsteps, energy_every,
                                     rec), self._ctx)
        if raw_records:
            return p, v, np.ctypeslib.as_array(rec)[:nsteps]
        return p, v, [rec[i].as_dict() for i in range(nsteps)]

    # ---- observation ----
    def thermo(self):
        t = Thermo()
        _check(library().md_get_thermo(self._ctx, C.byref(t)), self._ctx)
        return t.as_dict()

    def history(self, n):
        buf = (Thermo * max(n, 1))()
        got = C.c_int()
        _check(library().md_get_thermo_history(self._ctx, buf, n, C.byref(got)), self._ctx)
        return [buf[i].as_dict() for i in range(got.value)]

    def info(self):
        i = Info()
        _check(library().md_get_info(self._ctx, C.byref(i)), self._ctx)
        return {"natom": i.natom, "pitch": i.pitch, "capacity": i.capacity,
                "ncell": list(i.ncell), "stencil": list(i.stencil), "binlen": list(i.binlen),
                "pair_tpa": i.pair_threads_per_atom, "list_tpa": i.list_threads_per_atom,
                "builds": i.builds, "max_neighbors": i.max_neighbors,
                "kernels_per_step": i.kernels_per_step,
                "kernels_per_rebuild": i.kernels_per_rebuild,
                "kernels_per_graph": i.kernels_per_graph,
                "pair_depth": i.pair_entries_per_lane,
                "centered": bool(i.positions_centered),
                "fused_step": bool(i.fused_step), "rebuild_inline": bool(i.rebuild_inline),
                "list_regrows": i.list_regrows, "cell_regrids": i.cell_regrids,
                "pme_grid": list(i.pme_grid)}

    def neighbor_list(self, nmax):
        """Reference layout (neighborlist.cu:284): (nnlist[pitch*nmax], nnlist_max[pitch])."""
        pitch = ((self.natom + 255) // 256) * 256
        nn = np.zeros(pitch * nmax, np.uint32)
        nm = np.zeros(pitch, np.uint32)
        _check(library().md_get_neighbor_list(self._ctx, nn.ctypes.data, nm.ctypes.data, pitch, nmax),
               self._ctx)
        return nn, nm

    def order(self):
        p = np.zeros(self.natom, np.int32)
        _check(library().md_get_order(self._ctx, p.ctypes.data), self._ctx)
        return p

    def cell_ranks(self):
        info = self.info()
        r = np.zeros(int(np.prod(info["ncell"])), np.int32)
        _check(library().md_get_cell_ranks(self._ctx, r.ctypes.data), self._ctx)
        return r

    def time_pair(self, nrep=20):
        """Average ms per launch of the pair kernel (CUDA events, own stream)."""
        ms = C.c_float()
        _check(library().md_time_pair(self._ctx, nrep, C.byref(ms)), self._ctx)
        return ms.value

    def time_rebuild(self, nrep=10):
        """Average ms of a full list build (CUDA events, own stream)."""
        ms = C.c_float()
        _check(library().md_time_rebuild(self._ctx, nrep, C.byref(ms)), self._ctx)
        return ms.value

    def autotune(self):
        """Pick the fastest pair / list-build variants; returns (pair_tpa, list_tpa)."""
        a, b = C.c_int(), C.c_int()
        _check(library().md_autotune(self._ctx, C.byref(a), C.byref(b)), self._ctx)
        return a.value, b.value

    def set_type_exclusions(self, mask):
        """mask[a] bit b: exclude all pairs of types a and b (0-based)."""
        m = np.ascontiguousarray(mask, np.uint32)
        _check(library().md_set_type_exclusions(self._ctx, m.ctypes.data), self._ctx)

    def set_graphs(self, use_graphs=True):
        """Replay captured step graphs (default) or launch eagerly."""
        _check(library().md_set_graphs(self._ctx, 1 if use_graphs else 0), self._ctx)

    def set_graph_rebuild(self, inline=True):
        """Step graphs: rebuild passes inline (True) or behind a conditional node."""
        _check(library().md_set_graph_rebuild(self._ctx, 1 if inline else 0), self._ctx)

    def set_precision(self, bits):
        """32: FP32 pair arithmetic (the default); 64: every force term in FP64
        on the FP64 positions (the plain FP64 form, for reference runs)."""
        _check(library().md_set_precision(self._ctx, int(bits)), self._ctx)

    def set_barostat(self, press_bar, tau_p_fs=1000.0, compressibility_per_bar=4.5e-5):
        """NPT contexts: the Berendsen barostat's target pressure (bar), time
        constant (fs) and compressibility (1/bar)."""
        _check(library().md_set_barostat(self._ctx, float(press_bar), float(tau_p_fs),
                                         float(compressibility_per_bar)), self._ctx)

    def set_pme(self, k0, k1=None, k2=None):
        """lkspace 2: the reciprocal Ewald sum by smooth particle-mesh Ewald on
        a k0 x k1 x k2 grid (multiples of 8, at least 16; 0: off)."""
        k1 = k0 if k1 is None else k1
        k2 = k0 if k2 is None else k2
        _check(library().md_set_pme(self._ctx, int(k0), int(k1), int(k2)), self._ctx)

    def replica_boxes(self):
        """(box edges (nrep, 3) in A, last-step pressures (nrep,) in bar)."""
        n = len(getattr(self, "replica_sizes", [self.natom]))
        box = np.zeros((n, 3))
        p = np.zeros(n)
        _check(library().md_get_replica_box(self._ctx, box.ctypes.data, p.ctypes.data, n), self._ctx)
        return box, p

    def set_fused_step(self, fused=True):
        """Leapfrog without bonded terms: pair forces and update in one kernel."""
        _check(library().md_set_fused_step(self._ctx, 1 if fused else 0), self._ctx)

    def set_tuning(self, pair_tpa, list_tpa, pair_depth=0):
        _check(library().md_set_tuning(self._ctx, pair_tpa, list_tpa), self._ctx)
        if pair_depth:
            _check(library().md_set_pair_depth(self._ctx, pair_depth), self._ctx)

    def write_cfg(self, path):
        _check(library().md_write_cfg(self._ctx, path.encode()), self._ctx)

    def write_xyz(self, path, append=False):
        """One XYZ frame (full precision); append=True builds a trajectory."""
        _check(library().md_write_xyz(self._ctx, path.encode(), 1 if append else 0), self._ctx)

    def write_restart(self, path):
        """The exact state of a single system (FP64 positions and velocities,
        step count, thermostat state)."""
        _check(library().md_write_restart(self._ctx, path.encode()), self._ctx)

    def read_restart(self, path):
        """Load a restart of the same system; the list is rebuilt."""
        _check(library().md_read_restart(self._ctx, path.encode()), self._ctx)
