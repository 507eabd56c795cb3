"""The GPU adjoint (md_adjoint_run) against the oracle's FP64 adjoint and
FP64 central finite differences.

Tolerances (stated):
* loss: 1e-5 relative (FP32 forces vs FP64 over a short trajectory);
* gradients: 1e-3 relative to the largest component of each group (lj1
  entries, lj2 entries, charge scale), against the FP64 adjoint and against
  FP64 central differences (h = 1e-5 relative);
* a replica's loss and gradient do not depend on the batch it runs in
  (bit-exact) and barely on the checkpoint interval (loss 1e-7, gradients
  1e-5: list builds forced at other frames change the FP32 summation order).
"""
import numpy as np
import pytest

import oracle
from md_gpu_gb300 import MDSystem, synth
from md_gpu_gb300 import build as mdbuild

pytestmark = pytest.mark.gpu

NBINS, DR, SIGMA = 150, 0.05, 0.05     # 7.5 A: inside the clamped cutoff of the small boxes
NSTEPS = 20


@pytest.fixture(scope="module", autouse=True)
def _lib():
    mdbuild.build()


def _arrays():
    out = []
    for n, seed in ((216, 3), (256, 4)):
        a = synth.to_arrays(synth.nacl_replica(n, seed=seed))
        a["integrator"] = 1      # velocity Verlet
        a["enstype"] = 0
        out.append(a)
    return out


def _problem(a, w_pe=1.0, w_rdf=1.0):
    return oracle.AdjProblem(
        box=a["box"].astype(float), itype=a["itype"], q=a["charge"].astype(float),
        mass=a["type_mass"].astype(float)[a["itype"]], lj1=a["lj1"].astype(float),
        lj2=a["lj2"].astype(float), x0=a["pos"].astype(float), v0=a["vel"].astype(float),
        rcutsq=a["rcutsq"], alfa=a["alfa"], dt=a["dt"], nsteps=NSTEPS, w_pe=w_pe, w_rdf=w_rdf,
        nbins=NBINS, rdf_dr=DR, rdf_sigma=SIGMA)


@pytest.fixture(scope="module")
def reference():
    arrs = _arrays()
    out = []
    for a in arrs:
        prob = _problem(a)
        _, g, _ = oracle.adj_loss(prob)
        target = 1.05 * g
        loss, d1, d2, dlns, gbar = oracle.adj_grad(prob, target)
        out.append(dict(prob=prob, target=target, loss=loss, d1=d1, d2=d2, dlns=dlns, gbar=gbar))
    return arrs, out


def _gpu(arrs, targets, checkpoint=8, gradient=True):
    with MDSystem.from_batch(arrs) as b:
        return b.adjoint(NSTEPS, checkpoint=checkpoint, nbins=NBINS, dr=DR, sigma=SIGMA,
                         target=np.stack(targets), gradient=gradient)


def _close(a, b, rel):
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= rel * scale


def test_gpu_adjoint_matches_fp64_adjoint(reference):
    arrs, ref = reference
    out = _gpu(arrs, [r["target"] for r in ref])
    for k, r in enumerate(ref):
        assert abs(out["loss"][k] - r["loss"]) <= 1e-5 * abs(r["loss"])
        assert _close(out["gbar"][k], r["gbar"], 1e-4)
        assert _close(out["dlj1"][k, :2, :2], r["d1"], 1e-3)
        assert _close(out["dlj2"][k, :2, :2], r["d2"], 1e-3)
        assert abs(out["dlns"][k] - r["dlns"]) <= 1e-3 * abs(r["dlns"])


def test_gpu_adjoint_matches_central_differences(reference):
    """FP64 central differences of the oracle's forward loss (h = 1e-5)."""
    arrs, ref = reference
    out = _gpu(arrs, [r["target"] for r in ref])
    r = ref[1]
    prob, tg = r["prob"], r["target"]
    h = 1e-5
    L = lambda **kw: oracle.adj_loss(prob, tg, **kw)[0]
    fd = (L(q=prob.q * np.exp(h)) - L(q=prob.q * np.exp(-h))) / (2 * h)
    assert abs(out["dlns"][1] - fd) <= 1e-3 * abs(fd)
    for kw, key in (("lj1", "dlj1"), ("lj2", "dlj2")):
        base = getattr(prob, kw)
        p, m = base.copy(), base.copy()
        dv = h * base[0, 1]
        p[0, 1] += dv; p[1, 0] += dv
        m[0, 1] -= dv; m[1, 0] -= dv
        fd = (L(**{kw: p}) - L(**{kw: m})) / (2 * dv)
        ad = out[key][1, 0, 1] + out[key][1, 1, 0]
        assert abs(ad - fd) <= 1e-3 * abs(fd), (kw, ad, fd)


def test_gpu_adjoint_replica_independent_of_batch(reference):
    arrs, ref = reference
    both = _gpu(arrs, [r["target"] for r in ref])
    alone = _gpu(arrs[1:], [ref[1]["target"]])
    assert both["loss"][1] == alone["loss"][0]
    assert np.array_equal(both["dlj1"][1], alone["dlj1"][0])
    assert np.array_equal(both["dlns"][1:], alone["dlns"])


def test_gpu_adjoint_checkpoint_interval(reference):
    arrs, ref = reference
    tg = [r["target"] for r in ref]
    a = _gpu(arrs, tg, checkpoint=5)
    b = _gpu(arrs, tg, checkpoint=50)
    # a different checkpoint interval forces list builds at other frames:
    # the list order, hence the FP32 summation order, differs
    assert np.abs(a["loss"] - b["loss"]).max() <= 1e-7 * np.abs(b["loss"]).max()
    for key in ("dlj1", "dlj2", "dlns"):
        assert _close(a[key], b[key], 1e-5)


def test_gpu_forward_only_and_final_state(reference):
    """gradient = 0 gives the same loss; the context ends at the last frame
    either way."""
    arrs, ref = reference
    tg = np.stack([r["target"] for r in ref])
    with MDSystem.from_batch(arrs) as b1, MDSystem.from_batch(arrs) as b2:
        f = b1.adjoint(NSTEPS, checkpoint=8, nbins=NBINS, dr=DR, sigma=SIGMA, target=tg, gradient=False)
        g = b2.adjoint(NSTEPS, checkpoint=8, nbins=NBINS, dr=DR, sigma=SIGMA, target=tg, gradient=True)
        assert np.array_equal(f["loss"], g["loss"])
        assert np.array_equal(b1.positions(), b2.positions())


def test_autograd_wrapper(reference):
    torch = pytest.importorskip("torch")
    from md_gpu_gb300.autograd import make_function
    arrs, ref = reference
    tg = np.stack([r["target"] for r in ref])
    base = arrs[0]

    def build(lj1, lj2, s):
        reps = []
        for a in arrs:
            reps.append(dict(a, lj1=lj1.astype(np.float32), lj2=lj2.astype(np.float32),
                             charge=(a["charge"] * s).astype(np.float32)))
        return MDSystem.from_batch(reps)

    fn = make_function()
    lj1 = torch.tensor(base["lj1"].astype(np.float64), requires_grad=True)
    lj2 = torch.tensor(base["lj2"].astype(np.float64), requires_grad=True)
    lns = torch.tensor(0.0, dtype=torch.float64, requires_grad=True)
    kw = dict(nsteps=NSTEPS, checkpoint=8, nbins=NBINS, dr=DR, sigma=SIGMA, target=tg)
    loss = fn.apply(lj1, lj2, lns, build, kw)
    loss.sum().backward()
    direct = _gpu(arrs, list(tg))
    assert np.allclose(loss.detach().numpy(), direct["loss"], rtol=0, atol=0)
    assert np.allclose(lj1.grad.numpy(), direct["dlj1"][:, :2, :2].sum(0), rtol=1e-12)
    assert np.isclose(lns.grad.item(), direct["dlns"].sum(), rtol=1e-12)


def test_gpu_adjoint_with_bonds_and_angles():
    """Flexible water replicas (harmonic bonds and angles, the bonded pairs
    excluded): loss (1e-4 relative), RDF and gradients (1e-3) against the
    oracle's FP64 adjoint (whose bonded part is checked against central
    differences on the CPU), and the charge-scale gradient against FP64
    central differences."""
    import golden_util as gu
    cases = [gu.water_adjoint(nside=6, seed=s, rc=8.0, nsteps=NSTEPS, nbins=NBINS, rdf_dr=DR,
                              rdf_sigma=SIGMA) for s in (7, 8)]
    refs = []
    for _, prob in cases:
        _, g, _ = oracle.adj_loss(prob)
        target = 1.05 * g
        refs.append((target,) + oracle.adj_grad(prob, target))
    with MDSystem.from_batch([a for a, _ in cases]) as b:
        out = b.adjoint(NSTEPS, checkpoint=8, nbins=NBINS, dr=DR, sigma=SIGMA,
                        target=np.stack([r[0] for r in refs]), gradient=True)
    for k, (target, loss, d1, d2, dlns, gbar) in enumerate(refs):
        # the loss is a small difference of large pair and bonded energies:
        # 1e-4 of it (~1e-5 kJ/mol per atom) covers the FP32 dynamics
        assert abs(out["loss"][k] - loss) <= 1e-4 * abs(loss), (out["loss"][k], loss)
        assert _close(out["gbar"][k], gbar, 1e-4)
        assert _close(out["dlj1"][k, :2, :2], d1, 1e-3), (out["dlj1"][k, :2, :2], d1)
        assert _close(out["dlj2"][k, :2, :2], d2, 1e-3), (out["dlj2"][k, :2, :2], d2)
        assert abs(out["dlns"][k] - dlns) <= 1e-3 * abs(dlns), (out["dlns"][k], dlns)
    prob, target = cases[1][1], refs[1][0]
    h = 1e-5
    L = lambda **kw: oracle.adj_loss(prob, target, **kw)[0]
    fd = (L(q=prob.q * np.exp(h)) - L(q=prob.q * np.exp(-h))) / (2 * h)
    assert abs(out["dlns"][1] - fd) <= 1e-3 * abs(fd)
