"""The oracle's FP64 adjoint of velocity Verlet (test infrastructure for the
GPU adjoint) against FP64 central finite differences of its own forward run.

Tolerance: 1e-4 relative per parameter (both are FP64; the difference is the
finite-difference truncation at h = 1e-5 relative and the LJ force step at
the cutoff, which the adjoint does not see)."""
import numpy as np
import pytest

import oracle
from md_gpu_gb300 import synth


def _problem(n=216, seed=3, nsteps=12, w_pe=1.0, w_rdf=1.0):
    a = synth.to_arrays(synth.nacl_replica(n, seed=seed))
    return oracle.AdjProblem(
        box=a["box"].astype(float), itype=a["itype"], q=a["charge"].astype(float),
        mass=a["type_mass"].astype(float)[a["itype"]], lj1=a["lj1"].astype(float),
        lj2=a["lj2"].astype(float), x0=a["pos"].astype(float), v0=a["vel"].astype(float),
        rcutsq=a["rcutsq"], alfa=a["alfa"], dt=2.0, nsteps=nsteps, w_pe=w_pe, w_rdf=w_rdf)


@pytest.mark.parametrize("w_pe,w_rdf", [(1.0, 0.0), (0.0, 1.0), (1.0, 1.0)])
def test_adjoint_matches_finite_differences(w_pe, w_rdf):
    prob = _problem(w_pe=w_pe, w_rdf=w_rdf)
    _, g, _ = oracle.adj_loss(prob)
    target = 1.05 * g
    loss, d1, d2, dlns, _ = oracle.adj_grad(prob, target)
    h = 1e-5

    def L(**kw):
        return oracle.adj_loss(prob, target, **kw)[0]

    checks = []
    for kw, a, b in [("lj1", 0, 1), ("lj1", 1, 1), ("lj2", 0, 0), ("lj2", 0, 1)]:
        base = getattr(prob, kw)
        p, m = base.copy(), base.copy()
        dv = h * base[a, b]
        p[a, b] += dv
        m[a, b] -= dv
        if a != b:
            p[b, a] += dv
            m[b, a] -= dv
        fd = (L(**{kw: p}) - L(**{kw: m})) / (2 * dv)
        dd = d1 if kw == "lj1" else d2
        checks.append((fd, dd[a, b] + (dd[b, a] if a != b else 0.0)))
    fd = (L(q=prob.q * np.exp(h)) - L(q=prob.q * np.exp(-h))) / (2 * h)
    checks.append((fd, dlns))
    for fd, ad in checks:
        assert abs(fd - ad) <= 1e-4 * max(abs(fd), 1e-12 * abs(loss)), (fd, ad)


def test_adjoint_loss_is_forward_loss():
    prob = _problem(nsteps=5)
    l0, g, pe = oracle.adj_loss(prob)
    l1, _, _, _, g1 = oracle.adj_grad(prob)
    assert l0 == l1
    assert np.array_equal(g, g1)
    assert abs(l0 - (pe / len(prob.itype) + (g * g).sum())) <= 1e-9 * abs(l0)


def test_lorentz_berthelot_chain_rule():
    """Table-entry gradients mapped to per-type eps and sigma agree with
    central differences in eps / sigma space."""
    from md_gpu_gb300 import params
    prob = _problem(nsteps=8)
    eps = np.array([0.13, 0.10]) * 4.184
    sig = np.array([2.35, 4.40])
    l1, l2 = params.lb_tables(eps, sig)
    prob.lj1, prob.lj2 = l1, l2
    _, g, _ = oracle.adj_loss(prob)
    tg = 1.05 * g
    _, d1, d2, _, _ = oracle.adj_grad(prob, tg)
    de, ds = params.lb_chain(d1, d2, eps, sig)
    h = 1e-6
    for k in range(2):
        for arr, ad in ((eps, de), (sig, ds)):
            p, m = arr.copy(), arr.copy()
            p[k] *= 1 + h
            m[k] *= 1 - h
            if arr is eps:
                lp, lm = params.lb_tables(p, sig), params.lb_tables(m, sig)
            else:
                lp, lm = params.lb_tables(eps, p), params.lb_tables(eps, m)
            fd = (oracle.adj_loss(prob, tg, lj1=lp[0], lj2=lp[1])[0] -
                  oracle.adj_loss(prob, tg, lj1=lm[0], lj2=lm[1])[0]) / (2 * h * arr[k])
            assert abs(fd - ad[k]) <= 1e-4 * abs(fd), (k, fd, ad[k])


def test_adjoint_with_bonds_and_angles_matches_finite_differences():
    """Flexible water (bonds, angles, the bonded pairs excluded from the pair
    terms and the RDF): the adjoint, whose bonded J w is a central difference
    of the bonded forces along w, against central differences of the loss."""
    import golden_util as gu
    _, prob = gu.water_adjoint(nside=4, seed=5, rc=5.0, nsteps=12, nbins=80, rdf_dr=0.05, rdf_sigma=0.05)
    _, g, _ = oracle.adj_loss(prob)
    target = 1.05 * g
    loss, d1, d2, dlns, _ = oracle.adj_grad(prob, target)
    h = 1e-5
    L = lambda **kw: oracle.adj_loss(prob, target, **kw)[0]
    fd = (L(q=prob.q * np.exp(h)) - L(q=prob.q * np.exp(-h))) / (2 * h)
    assert abs(fd - dlns) <= 1e-4 * abs(fd), (fd, dlns)
    for kw, dd in (("lj1", d1), ("lj2", d2)):
        base = getattr(prob, kw)
        p, m = base.copy(), base.copy()
        dv = h * base[0, 0]
        p[0, 0] += dv
        m[0, 0] -= dv
        fd = (L(**{kw: p}) - L(**{kw: m})) / (2 * dv)
        assert abs(fd - dd[0, 0]) <= 1e-4 * abs(fd), (kw, fd, dd[0, 0])
