"""The adjoint at the check size of the differentiable-MD configuration: one
512-ion NaCl replica (1.5 g/cm^3, 1200 K; the cutoff clamped to 11.73 A so
that cutoff + skin stays inside half the 25.5 A box), velocity Verlet NVE at
dt 2 fs, loss = <U>/N + sum_b (gbar_b - target_b)^2 of the Gaussian-smoothed
Na-Cl RDF (200 bins of 0.05 A, sigma 0.05 A), the target made by the same
FP64 forward run at eps, sigma and charges +5%.

Horizon: 100 steps (0.2 ps) with checkpoints every 50 steps (two recompute
segments).  Over the full 2000-step horizon finite differences leave the
linear regime (chaos), so the check is made on this horizon.

Gradients with respect to the five physical parameters (eps_Na, sigma_Na,
eps_Cl, sigma_Cl under Lorentz-Berthelot mixing, and the charge scale), each
within 1e-3 relative of (a) the oracle's FP64 adjoint mapped by the same
chain rule and (b) FP64 central differences of the oracle's forward loss
with h = 1e-4 relative (the LJ tables rebuilt from the perturbed per-type
parameters); the FP64 adjoint itself agrees with the central differences to
1e-4.
"""
import numpy as np
import pytest

import oracle
from md_gpu_gb300 import MDSystem, params, synth
from md_gpu_gb300 import build as mdbuild

pytestmark = pytest.mark.gpu

NATOM, NSTEPS, CKPT = 512, 100, 50
NBINS, DR, SIGMA = 200, 0.05, 0.05
H = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _lib():
    mdbuild.build()


@pytest.fixture(scope="module")
def setup():
    eps = np.array([synth.NACL_LJ["Na"][1], synth.NACL_LJ["Cl"][1]]) * synth.KCAL
    sig = np.array([synth.NACL_LJ["Na"][0], synth.NACL_LJ["Cl"][0]])
    a = synth.to_arrays(synth.nacl_replica(NATOM, seed=21, integrator="vv", ensemble="nve"))
    l1, l2 = params.lb_tables(eps, sig)
    a.update(lj1=l1.astype(np.float32), lj2=l2.astype(np.float32))
    q0 = a["charge"].astype(np.float64)

    def problem(e, s, qscale):
        t1, t2 = params.lb_tables(e, s)
        return oracle.AdjProblem(
            box=a["box"].astype(float), itype=a["itype"], q=q0 * qscale,
            mass=a["type_mass"].astype(float)[a["itype"]], lj1=t1, lj2=t2, x0=a["pos"].astype(float),
            v0=a["vel"].astype(float), rcutsq=a["rcutsq"], alfa=a["alfa"], dt=a["dt"], nsteps=NSTEPS,
            nbins=NBINS, rdf_dr=DR, rdf_sigma=SIGMA)

    target = oracle.adj_loss(problem(eps * 1.05, sig * 1.05, 1.05))[1]
    base = problem(eps, sig, 1.0)
    loss, d1, d2, dlns, _ = oracle.adj_grad(base, target)
    de, ds = params.lb_chain(d1, d2, eps, sig)
    fp64_adj = np.array([de[0], ds[0], de[1], ds[1], dlns])

    # FP64 central differences of the forward loss, h = 1e-4 relative
    L = lambda e, s, qs: oracle.adj_loss(problem(e, s, qs), target)[0]
    fd = []
    for t in range(2):
        for which in ("eps", "sig"):
            v = eps if which == "eps" else sig
            dv = H * v[t]
            p, m = v.copy(), v.copy()
            p[t] += dv
            m[t] -= dv
            if which == "eps":
                fd.append((L(p, sig, 1.0) - L(m, sig, 1.0)) / (2 * dv))
            else:
                fd.append((L(eps, p, 1.0) - L(eps, m, 1.0)) / (2 * dv))
    fd.append((L(eps, sig, np.exp(H)) - L(eps, sig, np.exp(-H))) / (2 * H))
    return dict(a=a, eps=eps, sig=sig, target=target, loss=loss, fp64_adj=fp64_adj, fd=np.array(fd))


def _gpu(s):
    with MDSystem.from_batch([s["a"]]) as b:
        out = b.adjoint(NSTEPS, checkpoint=CKPT, nbins=NBINS, dr=DR, sigma=SIGMA, target=s["target"][None, :])
    de, ds = params.lb_chain(out["dlj1"][0], out["dlj2"][0], s["eps"], s["sig"])
    return out["loss"][0], np.array([de[0], ds[0], de[1], ds[1], out["dlns"][0]])


def test_fp64_adjoint_matches_central_differences(setup):
    rel = np.abs(setup["fp64_adj"] - setup["fd"]) / np.abs(setup["fd"])
    assert (rel <= 1e-4).all(), rel


def test_gpu_adjoint_five_parameters_n512(setup):
    loss, g = _gpu(setup)
    assert abs(loss - setup["loss"]) <= 1e-5 * abs(setup["loss"])
    rel_adj = np.abs(g - setup["fp64_adj"]) / np.abs(setup["fp64_adj"])
    rel_fd = np.abs(g - setup["fd"]) / np.abs(setup["fd"])
    print("gradients (eps_Na, sig_Na, eps_Cl, sig_Cl, ln q):", g, "rel vs FP64 adjoint", rel_adj,
          "rel vs central differences", rel_fd)
    assert (rel_adj <= 1e-3).all(), rel_adj
    assert (rel_fd <= 1e-3).all(), rel_fd
