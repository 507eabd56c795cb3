"""FP64 Ewald sums in numpy: the smooth particle-mesh Ewald (SPME) reciprocal
part that the library's PME kernels compute, and the exact Ewald reciprocal
sum over k-vectors that pins it.

TEST INFRASTRUCTURE ONLY: imported by tests/ (and bench.py's check of the
PME leg) as the checker; the product never imports it.

The reference carries SPME only as an unbuilt copy of GROMACS's pme.c
(src/pme.c: make_bsplines :1222, make_bspline_moduli :1297, spread_q_bsplines
:829, solve_pme :941, gather_f_bsplines :1136) and its lkspace 2 ("Ewald",
simulation.cu:91-95) computes the real-space term only.  This restates the
published method (Essmann et al., J. Chem. Phys. 103, 8577 (1995)) with
cubic (order 4) cardinal B-splines, in the grid convention the library uses:

    u_d = K_d * frac((x_d + L_d / 2) * (1 / L_d)),   i0 = floor(u_d),   w = u_d - i0
    points i0 - 3 + j (j = 0..3, periodic) with weights M4(w + 3 - j)
    Q(k) = sum_i q_i theta_x theta_y theta_z
    E_rec = 1/2 QFAC sum_m B(m) C(m) |DFT(Q)(m)|^2,
    C(m) = exp(-pi^2 |m|^2 / alpha^2) / (pi V |m|^2),  C(0) = 0,
    B(m) = prod_d 1 / ((2 + cos(2 pi m_d / K_d)) / 3)^2     (order 4)
    conv = unnormalised inverse DFT of B C DFT(Q)
    phi_i = sum_points theta theta theta conv,   E_rec = 1/2 QFAC sum_i q_i phi_i
    F_i,d = -QFAC q_i (K_d / L_d) sum_points dtheta_d theta theta conv

plus the self term -QFAC alpha / sqrt(pi) sum q^2, the neutralising
background -QFAC pi (sum q)^2 / (2 V alpha^2) and, for excluded pairs (which
the reciprocal sum includes), -QFAC q_i q_j erf(alpha r) / r.
"""
from __future__ import annotations

import math

import numpy as np

QFAC = 1389.35427611722   # e^2 / (4 pi eps0) in kJ/mol A (pair_forces.cu's qfac)


def bspline4(w):
    """Cubic B-spline weights of the 4 points i0-3 .. i0 and their
    derivatives with respect to u, for fractional offsets w in [0, 1)."""
    w = np.asarray(w, np.float64)
    t = np.stack([(1.0 - w) ** 3 / 6.0,
                  (3.0 * w ** 3 - 6.0 * w ** 2 + 4.0) / 6.0,
                  (-3.0 * w ** 3 + 3.0 * w ** 2 + 3.0 * w + 1.0) / 6.0,
                  w ** 3 / 6.0], -1)
    d = np.stack([-(1.0 - w) ** 2 / 2.0,
                  (3.0 * w ** 2 - 4.0 * w) / 2.0,
                  (-3.0 * w ** 2 + 2.0 * w + 1.0) / 2.0,
                  w ** 2 / 2.0], -1)
    return t, d


def grid_coords(pos, box, K):
    """(i0 (N, 3) int, w (N, 3)) of the library's grid convention."""
    pos = np.asarray(pos, np.float64)
    box = np.asarray(box, np.float64)
    K = np.asarray(K)
    t = (pos + 0.5 * box) * (1.0 / box)
    t -= np.floor(t)
    u = K * t
    i0 = np.floor(u).astype(np.int64)
    w = u - i0
    i0 %= K
    return i0, w


def influence(box, K, alpha):
    """B(m) C(m) on the half spectrum (K1, K2, K3 // 2 + 1) of a real DFT."""
    box = np.asarray(box, np.float64)
    V = float(np.prod(box))
    m = [np.fft.fftfreq(K[0], 1.0 / K[0]), np.fft.fftfreq(K[1], 1.0 / K[1]),
         np.fft.rfftfreq(K[2], 1.0 / K[2])]
    mod = [((2.0 + np.cos(2.0 * np.pi * m[d] / K[d])) / 3.0) ** 2 for d in range(3)]
    mx = (m[0] / box[0])[:, None, None]
    my = (m[1] / box[1])[None, :, None]
    mz = (m[2] / box[2])[None, None, :]
    m2 = mx * mx + my * my + mz * mz
    with np.errstate(divide="ignore", invalid="ignore"):
        c = np.exp(-np.pi ** 2 * m2 / alpha ** 2) / (np.pi * V * m2)
    c[0, 0, 0] = 0.0
    return c / (mod[0][:, None, None] * mod[1][None, :, None] * mod[2][None, None, :])


def spme_recip(pos, q, box, K, alpha):
    """SPME reciprocal part: (energy, forces (N, 3), per-atom energies (N,)),
    kJ/mol and kJ/mol/A, FP64."""
    pos = np.asarray(pos, np.float64)
    q = np.asarray(q, np.float64)
    K = tuple(int(k) for k in K)
    n = len(q)
    i0, w = grid_coords(pos, box, K)
    th, dth = [], []
    for d in range(3):
        t, dt = bspline4(w[:, d])
        th.append(t)
        dth.append(dt)
    idx = [(i0[:, d, None] - 3 + np.arange(4)[None, :]) % K[d] for d in range(3)]
    Q = np.zeros(K)
    for a in range(4):
        for b in range(4):
            wab = q * th[0][:, a] * th[1][:, b]
            for c in range(4):
                np.add.at(Q, (idx[0][:, a], idx[1][:, b], idx[2][:, c]), wab * th[2][:, c])
    F = np.fft.rfftn(Q)
    conv = np.fft.irfftn(F * influence(box, K, alpha), s=K) * float(np.prod(K))
    phi = np.zeros(n)
    g = np.zeros((n, 3))
    for a in range(4):
        for b in range(4):
            for c in range(4):
                v = conv[idx[0][:, a], idx[1][:, b], idx[2][:, c]]
                phi += th[0][:, a] * th[1][:, b] * th[2][:, c] * v
                g[:, 0] += dth[0][:, a] * th[1][:, b] * th[2][:, c] * v
                g[:, 1] += th[0][:, a] * dth[1][:, b] * th[2][:, c] * v
                g[:, 2] += th[0][:, a] * th[1][:, b] * dth[2][:, c] * v
    kl = np.asarray(K, np.float64) / np.asarray(box, np.float64)
    f = -QFAC * q[:, None] * kl[None, :] * g
    e_atom = 0.5 * QFAC * q * phi
    return float(e_atom.sum()), f, e_atom


def ewald_recip_exact(pos, q, box, alpha, kmax):
    """Exact Ewald reciprocal sum over m = (i/Lx, j/Ly, k/Lz), |i|,|j|,|k| <=
    kmax, m != 0: (energy, forces (N, 3)), FP64.  Small systems only."""
    pos = np.asarray(pos, np.float64)
    q = np.asarray(q, np.float64)
    box = np.asarray(box, np.float64)
    V = float(np.prod(box))
    r = np.arange(-kmax, kmax + 1)
    mi = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)
    mi = mi[np.any(mi != 0, axis=1)]
    m = mi / box[None, :]
    m2 = (m * m).sum(1)
    g = np.exp(-np.pi ** 2 * m2 / alpha ** 2) / m2
    energy = 0.0
    f = np.zeros_like(pos)
    for s in range(0, len(m), 512):
        ms, gs = m[s:s + 512], g[s:s + 512]
        ph = 2.0 * np.pi * pos @ ms.T                     # (N, M)
        e = np.exp(1j * ph)
        S = (q[:, None] * e).sum(0)                       # (M,)
        energy += float((gs * np.abs(S) ** 2).sum())
        im = np.imag(np.conj(S)[None, :] * e)             # (N, M)
        f += (2.0 * np.pi * q[:, None]) * ((im * gs[None, :]) @ ms)
    energy *= QFAC / (2.0 * np.pi * V)
    f *= QFAC / (np.pi * V)
    return energy, f


def self_energy(q, alpha):
    q = np.asarray(q, np.float64)
    return -QFAC * alpha / math.sqrt(math.pi) * float((q * q).sum())


def background_energy(q, box, alpha):
    """Energy of the neutralising background of a net charge."""
    qt = float(np.sum(q))
    return -QFAC * math.pi * qt * qt / (2.0 * float(np.prod(box)) * alpha * alpha)


def excluded_correction(pos, q, box, alpha, excl):
    """Removes each atom's excluded partners from the reciprocal sum, seen
    from that atom (as its list row omits them): for every j in excl[i],
    the force on i of -QFAC q_i q_j erf(alpha r) / r and half its energy;
    a pair excluded from both sides therefore counts once.  Minimum image.
    Returns (energy, forces (N, 3))."""
    pos = np.asarray(pos, np.float64)
    box = np.asarray(box, np.float64)
    f = np.zeros_like(pos)
    e = 0.0
    for i, js in enumerate(excl):
        for j in js:
            d = pos[i] - pos[j]
            d -= box * np.rint(d / box)
            r = math.sqrt(float(d @ d))
            qq = QFAC * q[i] * q[j]
            erf = math.erf(alpha * r)
            e -= 0.5 * qq * erf / r
            # F_i = -dE/dr d/r with E = -qq erf(ar)/r
            f[i] += qq * (2.0 * alpha / math.sqrt(math.pi) * math.exp(-alpha * alpha * r * r) * r - erf) / r ** 3 * d
    return e, f


def ewald_real(pos, q, box, alpha, rc, excluded=()):
    """Real-space Ewald term over all pairs within rc (minimum image), without
    an energy shift: (energy, forces (N, 3)), FP64, O(N^2)."""
    pos = np.asarray(pos, np.float64)
    q = np.asarray(q, np.float64)
    box = np.asarray(box, np.float64)
    n = len(q)
    ex = set((min(i, j), max(i, j)) for i, j in excluded)
    f = np.zeros_like(pos)
    e = 0.0
    from scipy.special import erfc
    for i in range(n - 1):
        d = pos[i] - pos[i + 1:]
        d -= box * np.rint(d / box)
        r2 = (d * d).sum(1)
        js = np.nonzero(r2 < rc * rc)[0]
        if ex:
            js = np.array([j for j in js if (i, i + 1 + j) not in ex], np.int64)
        if len(js) == 0:
            continue
        r = np.sqrt(r2[js])
        qq = QFAC * q[i] * q[i + 1 + js]
        ec = erfc(alpha * r)
        e += float((qq * ec / r).sum())
        fr = qq * (ec / r + 2.0 * alpha / math.sqrt(math.pi) * np.exp(-alpha * alpha * r * r)) / (r * r)
        fv = fr[:, None] * d[js]
        f[i] += fv.sum(0)
        np.add.at(f, i + 1 + js, -fv)
    return e, f
