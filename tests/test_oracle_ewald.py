"""The FP64 Ewald oracle (oracle/ewald.py) against itself and the exact sum,
on the CPU.  The reference has no working reciprocal-space code (its pme.c
is an unbuilt GROMACS copy), so the oracle's SPME is pinned to the exact
Ewald sum over k-vectors and to the Ewald identities:

* SPME converges to the exact reciprocal sum as the grid is refined;
* its energy is the same from the spectrum (1/2 sum B C |DFT Q|^2) and from
  the per-atom potentials (1/2 sum q phi);
* the total Coulomb energy real + reciprocal + self does not depend on the
  splitting parameter alpha;
* the forces are minus the gradient of the energy (central differences);
* the excluded-pair term is the erf part of the Coulomb pair.
"""
import math

import numpy as np
import pytest

from oracle import ewald as ew
from md_gpu_gb300 import synth


@pytest.fixture(scope="module")
def ions():
    a = synth.to_arrays(synth.nacl_rocksalt(ncell=3, seed=3))   # 216 ions, L = 19.1 A
    return (a["pos"].astype(np.float64), a["charge"].astype(np.float64), a["box"].astype(np.float64))


def _rel(f, g):
    return float(np.sqrt(((f - g) ** 2).sum() / (g ** 2).sum()))


def test_spme_converges_to_the_exact_sum(ions):
    pos, q, box = ions
    e_ex, f_ex = ew.ewald_recip_exact(pos, q, box, 0.35, 14)
    errs = []
    for K in (16, 32, 48):
        e, f, _ = ew.spme_recip(pos, q, box, (K, K, K), 0.35)
        errs.append(_rel(f, f_ex))
        assert abs(e - e_ex) <= 0.02 * abs(e_ex)
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] <= 2e-4


def test_spme_energy_from_spectrum_and_potentials(ions):
    pos, q, box = ions
    K = (24, 24, 32)
    e, _, e_atom = ew.spme_recip(pos, q, box, K, 0.3)
    i0, w = ew.grid_coords(pos, box, K)
    Q = np.zeros(K)
    th = [ew.bspline4(w[:, d])[0] for d in range(3)]
    for a in range(4):
        for b in range(4):
            for c in range(4):
                np.add.at(Q, ((i0[:, 0] - 3 + a) % K[0], (i0[:, 1] - 3 + b) % K[1], (i0[:, 2] - 3 + c) % K[2]),
                          q * th[0][:, a] * th[1][:, b] * th[2][:, c])
    F = np.fft.rfftn(Q)
    wgt = np.full(F.shape[2], 2.0)
    wgt[0] = 1.0
    if K[2] % 2 == 0:
        wgt[-1] = 1.0
    e_spec = 0.5 * ew.QFAC * float((ew.influence(box, K, 0.3) * np.abs(F) ** 2 * wgt[None, None, :]).sum())
    assert abs(e - e_spec) <= 1e-10 * abs(e)
    assert abs(e_atom.sum() - e) <= 1e-10 * abs(e)


def test_total_coulomb_energy_does_not_depend_on_alpha(ions):
    pos, q, box = ions
    rc = 0.5 * box[0] * 0.999
    tot = []
    for alpha in (0.40, 0.50):   # erfc(alpha rc) <= 1e-7 at rc = 9.55 A
        er, _ = ew.ewald_real(pos, q, box, alpha, rc)
        ek, _ = ew.ewald_recip_exact(pos, q, box, alpha, 16)
        tot.append(er + ek + ew.self_energy(q, alpha))
    assert abs(tot[0] - tot[1]) <= 1e-6 * abs(tot[0])


def test_forces_are_minus_the_energy_gradient(ions):
    pos, q, box = ions
    K = (32, 32, 32)
    _, f, _ = ew.spme_recip(pos, q, box, K, 0.35)
    h = 1e-5
    for i, d in ((0, 0), (7, 1), (100, 2)):
        p1, p2 = pos.copy(), pos.copy()
        p1[i, d] += h
        p2[i, d] -= h
        e1 = ew.spme_recip(p1, q, box, K, 0.35)[0]
        e2 = ew.spme_recip(p2, q, box, K, 0.35)[0]
        assert abs(-(e1 - e2) / (2 * h) - f[i, d]) <= 1e-5 * np.abs(f).max()


def test_excluded_term_is_the_erf_part_of_the_pair():
    box = np.array([30.0, 30.0, 30.0])
    pos = np.array([[0.0, 0.0, 0.0], [1.1, 0.3, -0.2]])
    q = np.array([0.7, -0.4])
    alpha = 0.3
    e, f = ew.excluded_correction(pos, q, box, alpha, [[1], [0]])
    r = float(np.linalg.norm(pos[0] - pos[1]))
    assert e == pytest.approx(-ew.QFAC * q[0] * q[1] * math.erf(alpha * r) / r, rel=1e-12)
    h = 1e-6
    p1 = pos.copy()
    p1[0, 0] += h
    p2 = pos.copy()
    p2[0, 0] -= h
    fd = -(ew.excluded_correction(p1, q, box, alpha, [[1], [0]])[0] -
           ew.excluded_correction(p2, q, box, alpha, [[1], [0]])[0]) / (2 * h)
    assert f[0, 0] == pytest.approx(fd, rel=1e-6)
    assert np.allclose(f[0], -f[1])
