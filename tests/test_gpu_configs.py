"""GPU parity at the benchmark configurations' own shapes (seeded synthetic
data from ``synth.workload_config``), through the C ABI, against the FP64
oracle (NumPy) or its C restatement (``oracle/cpu_port``).

* nni512 -- 512 NNI candidates of a 1000-leaf Yule tree, 40 sites: the
  log-likelihood of EVERY candidate within 1e-6 relative of the C
  restatement (fast_em/calculations.py:456-504); 3 EM iterations of 32
  sampled candidates against its EM (logL 1e-6, nu / phi 1e-3).
* fixed250 -- one 250-leaf tree, 30 sites: negative_llh in both models
  (per-site 1e-6) and 50 EM iterations of each model against the oracle's
  EM over the same fixed iteration count (logL 1e-6); the fastEM EM to its
  own stopping rule (iterations within one, logL 1e-6).
* grad4096 -- one 4096-leaf tree, 100 sites: the adjoint's gradient in 32
  sampled branch lengths against FP64 central differences (h = 1e-4) of the
  C restatement's log-likelihood, in nu and phi against the Richardson
  extrapolation of the differences at h and h/2, 1e-3 relative; the
  recompute and stored-partials modes bitwise equal.
* large50k -- one 50,000-leaf tree, 300 sites: per-site and total
  log-likelihood of one inside pass within 1e-6 relative of the C
  restatement; size-independent properties of one E-step (the six expected
  counts of every non-root branch sum to the site count; one EM iteration
  does not lower the log-likelihood).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from laml_gb300 import problem as PB  # noqa: E402
from laml_gb300 import synth  # noqa: E402
from laml_gb300 import tune  # noqa: E402
from laml_gb300.autograd import log_likelihood as ag_llh  # noqa: E402
from oracle import cpu_port  # noqa: E402
from oracle import pmm_oracle as O  # noqa: E402

LLH_RTOL = 1e-6


def _prob(w, t, compat):
    tr = O.parse_tree(w.newicks[t], w.leaf_order)
    enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, compat=compat)
    return O.Problem(tr, enc, compat)


@pytest.fixture(scope="module")
def nni512():
    return synth.workload_config("nni512")


def test_nni512_every_candidate_llh(nni512):
    w = nni512
    G = tune.pick_group_sites(w)
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, group_sites=G,
                      nu=0.5, phi=0.5)
    llh = b.log_likelihood()
    assert len(llh) == 512
    ref = cpu_port.loglik(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5)
    rel = np.abs(llh / ref - 1.0)
    assert rel.max() < LLH_RTOL, (int(rel.argmax()), float(rel.max()))
    # the generating parameters too
    b.set_params(nu=np.full(512, 0.1), phi=np.full(512, 0.15))
    llh = b.log_likelihood()
    ref = cpu_port.loglik(w.newicks, w.rows, w.Q, w.leaf_order, 0.1, 0.15)
    rel = np.abs(llh / ref - 1.0)
    assert rel.max() < LLH_RTOL, (int(rel.argmax()), float(rel.max()))


def test_nni512_em_sample(nni512):
    w = nni512
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True,
                      group_sites=tune.pick_group_sites(w))
    res = b.run_em(max_iters=3, rel_tol=-1.0, chunk=1)
    pick = np.random.default_rng(1).choice(512, 32, replace=False)
    llh, nu, phi, ds, _ = cpu_port.em([w.newicks[i] for i in pick], w.rows, w.Q, w.leaf_order,
                                      0.5, 0.5, iters=3)
    for j, i in enumerate(pick):
        r = res[i]
        assert r.iterations == 3
        assert r.llh == pytest.approx(llh[j], rel=LLH_RTOL), i
        assert r.nu == pytest.approx(nu[j], rel=1e-3), i
        assert r.phi == pytest.approx(phi[j], rel=1e-3), i
        np.testing.assert_allclose(r.branch_lengths, ds[j], rtol=1e-3, atol=1e-5)


@pytest.fixture(scope="module")
def fixed250():
    return synth.workload_config("fixed250")


@pytest.mark.parametrize("compat", [True, False])
def test_fixed250_negative_llh(fixed250, compat):
    w = fixed250
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=compat, nu=0.1, phi=0.15,
                      clamp=False)
    llh = b.log_likelihood()[0]
    prob = _prob(w, 0, compat)
    ref, ref_site = O.log_likelihood(prob, prob.tree.branch_lengths, 0.1, 0.15)
    np.testing.assert_allclose(b.site_llh(0), ref_site, rtol=LLH_RTOL)
    assert -llh == pytest.approx(-ref, rel=LLH_RTOL)


@pytest.mark.parametrize("compat", [True, False])
def test_fixed250_em50(fixed250, compat):
    """50 EM iterations from the solver's start (nu = phi = 0.5), no stopping
    rule on either side."""
    w = fixed250
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=compat, nu=0.5, phi=0.5,
                      clamp=compat)
    r = b.run_em(max_iters=50, rel_tol=-1.0, chunk=10)[0]
    assert r.iterations == 50
    if compat:
        llh, nu, phi, ds, _ = cpu_port.em(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5,
                                          iters=50)
        assert r.llh == pytest.approx(llh[0], rel=LLH_RTOL)
        assert r.nu == pytest.approx(nu[0], rel=1e-3)
        assert r.phi == pytest.approx(phi[0], rel=1e-3)
    else:
        prob = _prob(w, 0, False)
        ref = O.em_exact(prob, prob.tree.branch_lengths, 0.5, 0.5, max_iters=50, stop=-1.0)
        assert r.llh == pytest.approx(ref.llh, rel=LLH_RTOL)
        assert r.nu == pytest.approx(ref.nu, rel=1e-3, abs=1e-6)
        assert r.phi == pytest.approx(ref.phi, rel=1e-3, abs=1e-6)


def test_fixed250_em_converged(fixed250):
    """fastEM's EM to its 1e-5 stopping rule (fast_em/laml.py:183)."""
    w = fixed250
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, nu=0.5, phi=0.5)
    r = b.run_em(max_iters=1000)[0]
    prob = _prob(w, 0, True)
    ref = O.em_compat(prob, prob.tree.branch_lengths, 0.5, 0.5)
    assert abs(r.iterations - ref.iterations) <= 1
    assert r.llh == pytest.approx(ref.llh, rel=LLH_RTOL)


def test_grad4096_adjoint_vs_central_differences():
    w = synth.workload_config("grad4096")
    nu, phi = 0.05, 0.1
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, nu=nu, phi=phi,
                      clamp=False)
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, compat=True)
    d = tr.branch_lengths.copy()
    assert len(d) == 8191

    def grad(recompute):
        dt = torch.tensor(d, dtype=torch.float64, device="cuda", requires_grad=True)
        nt = torch.tensor([nu], dtype=torch.float64, device="cuda", requires_grad=True)
        pt = torch.tensor([phi], dtype=torch.float64, device="cuda", requires_grad=True)
        llh = ag_llh(dt, nt, pt, b, recompute=recompute)
        llh.sum().backward()
        return (float(llh[0]), dt.grad.cpu().numpy(), float(nt.grad[0]), float(pt.grad[0]))

    llh, gd, gnu, gphi = grad(False)
    llh2, gd2, gnu2, gphi2 = grad(True)
    assert llh == llh2 and gnu == gnu2 and gphi == gphi2
    np.testing.assert_array_equal(gd, gd2)

    def f(dd=d, nn=nu, pp=phi):
        return float(cpu_port.site_loglik(w.newicks[0], w.rows, w.Q, w.leaf_order, nn, pp,
                                          d=dd, enc=enc).sum())
    assert llh == pytest.approx(f(), rel=LLH_RTOL)
    h = 1e-4
    rng = np.random.default_rng(0)
    for v in rng.choice(len(d), 32, replace=False):
        dp, dm = d.copy(), d.copy()
        dp[v] += h
        dm[v] -= h
        fd = (f(dd=dp) - f(dd=dm)) / (2 * h)
        assert gd[v] == pytest.approx(fd, rel=1e-3, abs=1e-3), v
    # nu and phi: Richardson's extrapolation of the central differences at h
    # and h/2.  The phi direction's third derivative is ~2 M / phi^3 (~1e8
    # here), so the plain difference at h = 1e-4 is off by ~h^2 f^(3) / 6
    # ~ 0.1 on a gradient of ~-72.6 (a sum of terms of ~6e5 that cancel):
    # -72.537 at h = 1e-4, -72.616 at 5e-5, -72.641 at 1e-5.
    def rich(g):
        d1 = (g(h) - g(-h)) / (2 * h)
        d2 = (g(h / 2) - g(-h / 2)) / h
        return (4 * d2 - d1) / 3
    fd_nu = rich(lambda e: f(nn=nu + e))
    fd_phi = rich(lambda e: f(pp=phi + e))
    assert gnu == pytest.approx(fd_nu, rel=1e-3)
    assert gphi == pytest.approx(fd_phi, rel=1e-3)


def test_large50k_llh_and_estep_properties():
    w = synth.workload_config("large50k")
    nu, phi = 0.1, 0.2
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, nu=nu, phi=phi,
                      clamp=False)
    assert b.trees[0].num_leaves == 50000
    b.e_step()
    torch.cuda.synchronize()
    b.check_device_error()
    llh = float(b.work["tr_llh"][0].item())
    site = b.site_llh(0)
    enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, compat=True)
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    ref_site = cpu_port.site_loglik(w.newicks[0], w.rows, w.Q, w.leaf_order, nu, phi,
                                    d=tr.branch_lengths, enc=enc)
    np.testing.assert_allclose(site, ref_site, rtol=LLH_RTOL)
    assert llh == pytest.approx(ref_site.sum(), rel=LLH_RTOL)
    # every non-root branch: the six expected transition counts are a
    # distribution over (parent state, child state) per site
    cnt, _ = b.counts_from_partials()
    root = int(tr.root)
    tot = np.delete(cnt.sum(axis=1), root)
    K = len(w.Q)
    np.testing.assert_allclose(tot, K, rtol=1e-4)
    # EM does not lower the log-likelihood
    b.mstep()
    b.branch_terms()
    b.inside(update_em=False)
    after = float(b.work["tr_llh"][0].item())
    assert after >= llh - 1e-9 * abs(llh)
