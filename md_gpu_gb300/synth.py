"""Seeded synthetic systems written in md_gpu's input grammar.

The reference reads a run as three whitespace files, ``<name>.inp`` (run
parameters, simulation.cu:58-105), ``<name>.fld`` (force field,
simulation.cu:144-264) and ``<name>.cfg`` (configuration,
simulation.cu:278-316).  The generators here build the benchmark systems in
those units (length A, time fs, mass g/mol, energy kJ/mol, charge e) and
write them in that grammar, so the reference's parser, the oracle and this
library all read the same text.

Systems
-------
* :func:`argon_fcc`     plain LJ argon, reduced units mapped to sigma = 1 A,
  eps = 1 kJ/mol, m = 1 g/mol (tau = 100 fs): 4 * n^3 atoms, rho* = 0.8442.
* :func:`nacl_rocksalt` molten NaCl at 1.5 g/cm^3, LJ + Wolf Coulomb,
  8 * n^3 ions on a rocksalt lattice; n = 20 gives the 64000-ion system.
* :func:`water_grid`    flexible 3-site water at 0.997 g/cm^3, n^3 molecules,
  O on a cubic grid with random orientations; the H-H pair is written as a
  bond of a zero-force-constant type so the reference's 1-2 exclusions cover
  every intramolecular pair.

LJ and bonded parameters given in kcal/mol are converted with 4.184 and the
reference's U = k (r - r0)^2 and U = k (theta - theta0)^2 conventions.
"""
from __future__ import annotations

import dataclasses
import os
from typing import Dict, List, Optional, Tuple

import numpy as np

KCAL = 4.184
RGAS = 8.314e-3          # kJ/mol/K, the reference's 1000/8.314 (integrator.cu:155)
AVOGADRO = 6.02214076e23


@dataclasses.dataclass
class System:
    """One run: parameters, force field and configuration."""

    name: str
    inp: Dict[str, object]
    types: List[Tuple[str, float, float]]          # (name, mass g/mol, charge)
    vdw: List[Tuple[int, int, str, float, float]]   # (i, j, "LJ", sigma, eps) 1-based
    bond_types: List[Tuple[float, float]]           # (k, r0) as written in .fld
    angle_types: List[Tuple[float, float]]          # (k, theta0 deg) as written
    bonds: np.ndarray                               # (nb, 3): type, i, j (1-based)
    angles: np.ndarray                              # (na, 4): type, i, j(centre), k
    box: np.ndarray                                 # (3,)
    itype: np.ndarray                               # (N,) 1-based
    charge: np.ndarray                              # (N,)
    pos: np.ndarray                                 # (N, 3) centred in [-L/2, L/2)
    vel: np.ndarray                                 # (N, 3) A/fs

    @property
    def natom(self) -> int:
        return int(self.pos.shape[0])


def _maxwell(rng, masses, temp):
    """Maxwell-Boltzmann velocities in A/fs with zero net momentum."""
    m4 = masses * 1.0e4
    sig = np.sqrt(RGAS * temp / m4)
    v = rng.standard_normal((masses.shape[0], 3)) * sig[:, None]
    p = (v * m4[:, None]).sum(0) / m4.sum()
    return v - p[None, :]


def _centre(pos, box):
    return pos - box[None, :] * np.floor(pos / box[None, :] + 0.5)


def argon_fcc(ncell: int = 10, seed: int = 1, nsteps: int = 1000,
              integrator: str = "vv", jitter: float = 0.02) -> System:
    """fcc LJ argon in reduced units (sigma = eps = m = 1), T* = 0.72,
    rc = 2.5, skin 0.3, dt = 0.005 tau = 0.5 fs, NVE.  Sites are displaced
    uniformly by up to +-jitter sigma so the lattice symmetry is broken."""
    rho = 0.8442
    a = (4.0 / rho) ** (1.0 / 3.0)
    L = a * ncell
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(*[np.arange(ncell)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pos = (g[:, None, :] + basis[None, :, :]).reshape(-1, 3) * a - 0.5 * L + 0.25 * a
    rng = np.random.default_rng(seed)
    n = pos.shape[0]
    pos = pos + rng.uniform(-jitter, jitter, pos.shape)
    masses = np.ones(n)
    temp = 0.72 / RGAS      # T* = 0.72 with eps = 1 kJ/mol
    box = np.full(3, L)
    return System(
        name="argon",
        inp=dict(ensemble="nve", times=(0, nsteps, max(1, nsteps // 10), 0.5), cutoff=(2.5, 0),
                 reacf=1.0, skin=(0.3, 128), rdel=0.02, integrator=integrator),
        types=[("Ar", 1.0, 0.0)],
        vdw=[(1, 1, "LJ", 1.0, 1.0)],
        bond_types=[], angle_types=[],
        bonds=np.zeros((0, 3), np.int64), angles=np.zeros((0, 4), np.int64),
        box=box, itype=np.ones(n, np.int64), charge=np.zeros(n),
        pos=_centre(pos, box), vel=_maxwell(rng, masses, temp))


NACL_LJ = {"Na": (2.35, 0.13), "Cl": (4.40, 0.10)}   # sigma A, eps kcal/mol


def nacl_params(eps_scale=(1.0, 1.0), sig_scale=(1.0, 1.0)):
    """Na/Cl LJ lines with Lorentz-Berthelot cross terms, eps in kJ/mol."""
    sN, eN = NACL_LJ["Na"]
    sC, eC = NACL_LJ["Cl"]
    sN *= sig_scale[0]; sC *= sig_scale[1]
    eN *= KCAL * eps_scale[0]; eC *= KCAL * eps_scale[1]
    return [(1, 1, "LJ", float(sN), float(eN)),
            (1, 2, "LJ", float(0.5 * (sN + sC)), float(np.sqrt(eN * eC))),
            (2, 2, "LJ", float(sC), float(eC))]


def nacl_rocksalt(ncell: int = 20, seed: int = 1, temp: float = 1200.0, density: float = 1.5,
                  rc: float = 12.0, skin: float = 1.0, alpha: float = 0.2, dt: float = 2.0,
                  nsteps: int = 10000, nmaxlist: int = 512, ensemble: str = "nvt",
                  integrator: str = "leapfrog", charge_scale: float = 1.0,
                  vdw: Optional[list] = None, jitter: float = 0.25) -> System:
    """Rocksalt NaCl (8 ncell^3 ions) scaled to `density` g/cm^3, LJ + Wolf.
    Ions are displaced uniformly by up to +-jitter A from their sites."""
    mNa, mCl = 22.98977, 35.4527
    n = 8 * ncell ** 3
    rho = density / ((mNa + mCl) / 2.0) * AVOGADRO * 1e-24     # ions / A^3
    L = (n / rho) ** (1.0 / 3.0)
    a = L / ncell
    na = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    cl = na + np.array([0.5, 0.0, 0.0])
    g = np.stack(np.meshgrid(*[np.arange(ncell)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pna = (g[:, None, :] + na[None]).reshape(-1, 3)
    pcl = (g[:, None, :] + cl[None]).reshape(-1, 3)
    pos = np.empty((n, 3))
    pos[0::2] = pna
    pos[1::2] = pcl
    pos = pos * a - 0.5 * L + 0.25 * a
    itype = np.empty(n, np.int64)
    itype[0::2] = 1
    itype[1::2] = 2
    charge = np.where(itype == 1, 1.0, -1.0) * charge_scale
    masses = np.where(itype == 1, mNa, mCl)
    rng = np.random.default_rng(seed)
    pos = pos + rng.uniform(-jitter, jitter, pos.shape)
    box = np.full(3, L)
    inp = dict(ensemble=ensemble, temper=temp, times=(0, nsteps, max(1, nsteps // 10), dt),
               cutoff=(rc, 1), alfa=alpha, skin=(skin, nmaxlist), rdel=0.02,
               integrator=integrator)
    return System(
        name="nacl", inp=inp,
        types=[("Na", mNa, 1.0), ("Cl", mCl, -1.0)],
        vdw=vdw if vdw is not None else nacl_params(),
        bond_types=[], angle_types=[],
        bonds=np.zeros((0, 3), np.int64), angles=np.zeros((0, 4), np.int64),
        box=box, itype=itype, charge=charge,
        pos=_centre(pos, box), vel=_maxwell(rng, masses, temp))


def nacl_replica(natom: int, seed: int = 1, temp: float = 1200.0, density: float = 1.5,
                 rc: float = 12.0, skin: float = 1.0, alpha: float = 0.2, dt: float = 2.0,
                 nsteps: int = 2000, nmaxlist: int = 416, eps_scale=(1.0, 1.0),
                 sig_scale=(1.0, 1.0), charge_scale: float = 1.0, integrator: str = "vv",
                 ensemble: str = "nve", jitter: float = 0.25) -> System:
    """NaCl-like replica of any even size.  natom ions at `density` g/cm^3
    occupy a random half-Na / half-Cl subset of the sites of a simple-cubic
    lattice with alternating site types (rocksalt) of m^3 >= natom sites,
    m even; ions are displaced by up to +-jitter A.  The cutoff is clamped to
    rc <= L/2 (1 - 1e-3) - skin so that cutoff + skin stays inside half the
    box (the minimum-image convention of the force and list kernels) for the
    smallest replicas; the clamped value is what the .inp carries."""
    natom = int(natom)
    if natom < 2 or natom % 2:
        raise ValueError("natom must be even and >= 2")
    mNa, mCl = 22.98977, 35.4527
    rho = density / ((mNa + mCl) / 2.0) * AVOGADRO * 1e-24
    L = (natom / rho) ** (1.0 / 3.0)
    m = int(np.ceil(natom ** (1.0 / 3.0) - 1e-9))
    m += m % 2
    a = L / m
    g = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)
    odd = g.sum(1) % 2 == 1
    rng = np.random.default_rng(seed)
    na_sites = rng.choice(np.flatnonzero(~odd), natom // 2, replace=False)
    cl_sites = rng.choice(np.flatnonzero(odd), natom // 2, replace=False)
    sites = np.empty(natom, np.int64)
    sites[0::2] = np.sort(na_sites)
    sites[1::2] = np.sort(cl_sites)
    pos = (g[sites] + 0.5) * a - 0.5 * L + rng.uniform(-jitter, jitter, (natom, 3))
    itype = np.empty(natom, np.int64)
    itype[0::2] = 1
    itype[1::2] = 2
    charge = np.where(itype == 1, 1.0, -1.0) * charge_scale
    masses = np.where(itype == 1, mNa, mCl)
    box = np.full(3, L)
    rc_eff = min(rc, 0.5 * L * (1.0 - 1e-3) - skin)
    inp = dict(ensemble=ensemble, temper=temp, times=(0, nsteps, max(1, nsteps // 10), dt),
               cutoff=(rc_eff, 1), alfa=alpha, skin=(skin, nmaxlist), rdel=0.02,
               integrator=integrator)
    return System(
        name="nacl", inp=inp,
        types=[("Na", mNa, 1.0), ("Cl", mCl, -1.0)],
        vdw=nacl_params(eps_scale=eps_scale, sig_scale=sig_scale),
        bond_types=[], angle_types=[],
        bonds=np.zeros((0, 3), np.int64), angles=np.zeros((0, 4), np.int64),
        box=box, itype=itype, charge=charge,
        pos=_centre(pos, box), vel=_maxwell(rng, masses, temp))


def nacl_melt64k() -> System:
    """The 64000-ion molten-NaCl benchmark system (nacl_rocksalt(ncell=20,
    seed=1) parameters) in its melted starting state at 1200 K, read from
    cases/nacl64k_melt.npz (made by cases/make_melt.py)."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cases", "nacl64k_melt.npz")
    z = np.load(path)
    base = nacl_rocksalt(ncell=int(z["ncell"]), seed=int(z["seed"]))
    return dataclasses.replace(base, pos=z["pos"].astype(np.float64), vel=z["vel"].astype(np.float64))


def replica_batch(nrep: int = 512, nmin: int = 256, nmax: int = 8192, seed: int = 1,
                  spread: float = 0.1, **kw) -> List[System]:
    """Uneven NaCl-like replicas: N uniform in [nmin, nmax] (rounded down to
    even), each with its own eps and sigma per type and charge scale drawn
    uniformly within +-spread of the molten-NaCl values; 1.5 g/cm^3, 1200 K."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(nrep):
        n = int(rng.integers(nmin, nmax + 1))
        n -= n % 2
        es = tuple(rng.uniform(1 - spread, 1 + spread, 2))
        ss = tuple(rng.uniform(1 - spread, 1 + spread, 2))
        qs = float(rng.uniform(1 - spread, 1 + spread))
        out.append(nacl_replica(n, seed=seed * 1000003 + r, eps_scale=es, sig_scale=ss,
                                charge_scale=qs, **kw))
    return out


def to_arrays(sys_: System) -> Dict[str, object]:
    """Keyword arguments of MDSystem.from_arrays for a system, with the unit
    conversions and float rounding of the reference's parser
    (simulation.cu:58-316): masses g/mol * 1e4, lj1 = 48 eps sigma^12,
    lj2 = 24 eps sigma^6, rc^2 in float, angles in rad."""
    f32 = np.float32
    p = sys_.inp
    nt = len(sys_.types)
    mass = np.array([f32(np.float64(f32(m)) * 10000.0) for (_, m, _) in sys_.types], f32)
    lj1 = np.zeros((nt, nt), f32)
    lj2 = np.zeros((nt, nt), f32)
    for (i, j, form, a, b) in sys_.vdw:
        a32, b32 = f32(a), f32(b)
        if form == "LJ":
            l1 = f32(np.float64(f32(48.0) * b32) * np.float64(a32) ** 12)
            l2 = f32(np.float64(f32(24.0) * b32) * np.float64(a32) ** 6)
        else:
            l1, l2 = f32(12.0) * a32, f32(6.0) * b32
        lj1[i - 1, j - 1] = lj1[j - 1, i - 1] = l1
        lj2[i - 1, j - 1] = lj2[j - 1, i - 1] = l2
    rc, lk = p["cutoff"]
    rc32 = f32(rc)
    integ = {"leapfrog": 0, "vv": 1, "nh": 2}[p.get("integrator", "leapfrog")]
    if len(sys_.bonds) or len(sys_.angles):
        raise ValueError("to_arrays: bonded systems are read from files")
    if lk == 0:
        eps = f32(p.get("reacf", 1.0))
        num = f32(2.0) * (eps - f32(1.0)) / (f32(2.0) * eps + f32(1.0))
        reacf, alfa = f32(np.float64(num) / np.float64(rc32) ** 3), f32(0.0)
    else:
        reacf, alfa = f32(0.0), f32(p["alfa"]) if lk == 1 else f32(3.09 / np.float64(rc32))
    return dict(box=sys_.box.astype(f32), itype=(sys_.itype - 1).astype(np.int32),
                charge=sys_.charge.astype(f32), pos=sys_.pos.astype(f32), vel=sys_.vel.astype(f32),
                type_mass=mass, lj1=lj1, lj2=lj2, lkspace=lk, rcutsq=float(rc32 * rc32),
                reacf=float(reacf), alfa=float(alfa), skin=float(f32(p["skin"][0])),
                nmaxlist=int(p["skin"][1]), dt=float(f32(p["times"][3])),
                enstype={"nve": 0, "nvt": 1, "npt": 2}[p["ensemble"]],
                temper_0=float(f32(p.get("temper", 0.0))), tau_t=float(f32(p.get("tau_t", 100.0))),
                integrator=integ)


def water_grid(nside: int = 32, seed: int = 1, temp: float = 300.0, rc: float = 10.0,
               skin: float = 1.0, alpha: float = 0.2, dt: float = 0.5, nsteps: int = 20000,
               nmaxlist: int = 768, integrator: str = "nh", h_jitter: float = 0.02) -> System:
    """Flexible 3-site water, nside^3 molecules at 0.997 g/cm^3.  Hydrogens
    are displaced uniformly by up to +-h_jitter A from the equilibrium
    geometry (thermal bond stretches are ~0.02 A at 300 K)."""
    mO, mH = 15.9994, 1.008
    nmol = nside ** 3
    rho_mol = 0.997 / (mO + 2 * mH) * AVOGADRO * 1e-24
    L = (nmol / rho_mol) ** (1.0 / 3.0)
    a = L / nside
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(nside)] * 3, indexing="ij"), -1).reshape(-1, 3)
    o = (g + 0.5) * a - 0.5 * L + rng.uniform(-0.1, 0.1, (nmol, 3))
    r0, th0 = 1.012, np.deg2rad(113.24)
    u = rng.standard_normal((nmol, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    w = rng.standard_normal((nmol, 3))
    w -= (w * u).sum(1, keepdims=True) * u
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    h1 = o + r0 * (np.cos(th0 / 2) * u + np.sin(th0 / 2) * w)
    h2 = o + r0 * (np.cos(th0 / 2) * u - np.sin(th0 / 2) * w)
    h1 = h1 + rng.uniform(-h_jitter, h_jitter, h1.shape)
    h2 = h2 + rng.uniform(-h_jitter, h_jitter, h2.shape)
    pos = np.empty((3 * nmol, 3))
    pos[0::3], pos[1::3], pos[2::3] = o, h1, h2
    itype = np.tile(np.array([1, 2, 2]), nmol)
    charge = np.where(itype == 1, -0.82, 0.41)
    masses = np.where(itype == 1, mO, mH)
    box = np.full(3, L)
    base = 3 * np.arange(nmol) + 1
    bonds = np.concatenate([
        np.stack([np.ones(nmol), base, base + 1], 1),
        np.stack([np.ones(nmol), base, base + 2], 1),
        np.stack([2 * np.ones(nmol), base + 1, base + 2], 1)]).astype(np.int64)
    order = np.argsort(np.concatenate([3 * np.arange(nmol), 3 * np.arange(nmol) + 1,
                                       3 * np.arange(nmol) + 2]), kind="stable")
    bonds = bonds[order]
    angles = np.stack([np.ones(nmol), base + 1, base, base + 2], 1).astype(np.int64)
    inp = dict(ensemble="nvt", temper=temp, times=(0, nsteps, max(1, nsteps // 10), dt),
               cutoff=(rc, 1), alfa=alpha, skin=(skin, nmaxlist), rdel=0.02,
               integrator=integrator)
    return System(
        name="water", inp=inp,
        types=[("O", mO, -0.82), ("H", mH, 0.41)],
        vdw=[(1, 1, "LJ", 3.166, 0.1554 * KCAL)],
        bond_types=[(1059.0 / 2 * KCAL, 1.012), (0.0, 1.0)],
        angle_types=[(75.9 / 2 * KCAL, 113.24)],
        bonds=bonds, angles=angles, box=box, itype=itype, charge=charge,
        pos=_centre(pos, box), vel=_maxwell(rng, masses, temp))


def write_case(sys_: System, directory: str, name: Optional[str] = None) -> str:
    """Write <name>.inp/.fld/.cfg in the reference grammar; returns the base path."""
    name = name or sys_.name
    os.makedirs(directory, exist_ok=True)
    base = os.path.join(directory, name)
    p = sys_.inp
    lines = [f"ensemble: {p['ensemble']}"]
    if p["ensemble"] == "nvt":
        lines.append(f"temper: {p['temper']!r}")
    elif p["ensemble"] == "npt":   # simulation.cu:71-75: T0 and P0 (bar)
        lines.append(f"temper: {p['temper']!r} {p.get('press', 1.0)!r}")
    t = p["times"]
    lines.append(f"times: {t[0]} {t[1]} {t[2]} {t[3]!r}")
    rc, lk = p["cutoff"]
    lines.append(f"cutoff: {rc!r} {lk}")
    if lk == 0:
        lines.append(f"reacf: {p.get('reacf', 1.0)!r}")
    elif lk == 1:
        lines.append(f"alfa: {p['alfa']!r}")
    else:
        lines.append(f"kmax: {p.get('kmax', 5)}")
    sk, nm = p["skin"]
    lines.append(f"skin: {sk!r} {nm}")
    lines.append(f"rdel: {p.get('rdel', 0.02)!r}")
    if "tau_t" in p:
        lines.append(f"tau_t: {p['tau_t']!r}")
    if "tau_p" in p:
        lines.append(f"tau_p: {p['tau_p']!r}")
    if "compressibility" in p:
        lines.append(f"compressibility: {p['compressibility']!r}")
    if "pme_spacing" in p:   # lkspace 2: the reciprocal Ewald sum on a grid of at most this spacing
        lines.append(f"pme_spacing: {p['pme_spacing']!r}")
    if p.get("integrator", "leapfrog") != "leapfrog":
        lines.append(f"integrator: {p['integrator']}")
    with open(base + ".inp", "w") as fh:
        fh.write("\n".join(lines) + "\n")

    n = sys_.natom
    counts = [int((sys_.itype == k + 1).sum()) for k in range(len(sys_.types))]
    out = [f"Atomtypes: {len(sys_.types)}"]
    for k, (nm_, m, q) in enumerate(sys_.types):
        out.append(f"{k + 1} {counts[k]}")
        out.append(f"{nm_} {m!r} {q!r}")
    out.append("")
    out.append(f"VDW_interactions: {len(sys_.vdw)}")
    for (i, j, form, a, b) in sys_.vdw:
        out.append(f"{i} {j} {form} {a!r} {b!r}")
    out.append("")
    out.append(f"Bond_types: {len(sys_.bond_types)}")
    for k, (kk, r0) in enumerate(sys_.bond_types):
        out.append(f"{k + 1} {kk!r} {r0!r}")
    out.append("")
    out.append(f"Angle_types: {len(sys_.angle_types)}")
    for k, (kk, th) in enumerate(sys_.angle_types):
        out.append(f"{k + 1} {kk!r} {th!r}")
    out.append("")
    out.append(f"Bonds: {len(sys_.bonds)}")
    out.extend(f"{k + 1} {b[0]} {b[1]} {b[2]}" for k, b in enumerate(sys_.bonds.tolist()))
    out.append("")
    out.append(f"Angles: {len(sys_.angles)}")
    out.extend(f"{k + 1} {a[0]} {a[1]} {a[2]} {a[3]}" for k, a in enumerate(sys_.angles.tolist()))
    with open(base + ".fld", "w") as fh:
        fh.write("\n".join(out) + "\n")

    L = sys_.box
    buf = [f"{n} 1", f"{L[0]:.9g} {L[1]:.9g} {L[2]:.9g}"]
    P, V, Q, T = sys_.pos, sys_.vel, sys_.charge, sys_.itype
    for i in range(n):
        buf.append(f"{i + 1} {T[i]} {Q[i]:.9g}")
        buf.append(f"{P[i, 0]:.9g} {P[i, 1]:.9g} {P[i, 2]:.9g}")
        buf.append(f"{V[i, 0]:.9g} {V[i, 1]:.9g} {V[i, 2]:.9g}")
    with open(base + ".cfg", "w") as fh:
        fh.write("\n".join(buf) + "\n")
    return base


CONFIGS = {
    "argon": lambda: argon_fcc(10),
    "nacl64k": lambda: nacl_rocksalt(20),
    "water": lambda: water_grid(32),
}
