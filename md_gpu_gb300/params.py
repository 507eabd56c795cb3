"""LJ parameters per atom type with Lorentz-Berthelot mixing, and the chain
rule from the library's table gradients to them.

The library differentiates with respect to the LJ table entries it uses,
lj1[a][b] = 48 eps_ab sigma_ab^12 and lj2[a][b] = 24 eps_ab sigma_ab^6 (the
reference's "LJ" form, simulation.cu:183-205), and the log of a common charge
scale.  With eps_ab = sqrt(eps_a eps_b) and sigma_ab = (sigma_a + sigma_b)/2
the gradient with respect to (eps_a, sigma_a) follows by the chain rule.
"""
from __future__ import annotations

import numpy as np


def lb_tables(eps, sig):
    """lj1, lj2 (ntype x ntype) from per-type eps (kJ/mol) and sigma (A)."""
    eps = np.asarray(eps, np.float64)
    sig = np.asarray(sig, np.float64)
    e = np.sqrt(np.outer(eps, eps))
    s = 0.5 * (sig[:, None] + sig[None, :])
    return 48.0 * e * s ** 12, 24.0 * e * s ** 6


def lb_chain(dlj1, dlj2, eps, sig):
    """d/d eps_a and d/d sigma_a from table-entry gradients dlj1[a][b],
    dlj2[a][b] (entry (a, b) as used by atoms of type a; both (a, b) and
    (b, a) depend on the same mixed pair)."""
    eps = np.asarray(eps, np.float64)
    sig = np.asarray(sig, np.float64)
    nt = len(eps)
    d1 = np.asarray(dlj1, np.float64)[:nt, :nt]
    d2 = np.asarray(dlj2, np.float64)[:nt, :nt]
    e = np.sqrt(np.outer(eps, eps))
    s = 0.5 * (sig[:, None] + sig[None, :])
    # derivatives of each entry with respect to eps_ab and sigma_ab
    g_e = d1 * 48.0 * s ** 12 + d2 * 24.0 * s ** 6
    g_s = d1 * 48.0 * e * 12.0 * s ** 11 + d2 * 24.0 * e * 6.0 * s ** 5
    deps = np.zeros(nt)
    dsig = np.zeros(nt)
    for a in range(nt):
        for b in range(nt):
            # eps_ab = sqrt(eps_a eps_b): d/d eps_a = eps_ab / (2 eps_a), twice on the diagonal
            de_a = e[a, b] / (2.0 * eps[a]) * (2.0 if a == b else 1.0)
            ds_a = 0.5 * (2.0 if a == b else 1.0)
            deps[a] += g_e[a, b] * de_a
            dsig[a] += g_s[a, b] * ds_a
            if a != b:
                deps[b] += g_e[a, b] * e[a, b] / (2.0 * eps[b])
                dsig[b] += g_s[a, b] * 0.5
    return deps, dsig
