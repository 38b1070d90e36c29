"""The hand-written adjoint (torch.autograd.Function) against central finite
differences of the FP64 oracle (h = 1e-4) and against the analytic gradient
of the reference's M-step objective (fast_em/laml.py:62-78) evaluated with
the oracle's expected counts.  Tolerance: 1e-3 relative (+1e-3 absolute)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from laml_gb300 import problem as PB  # noqa: E402
from laml_gb300 import synth  # noqa: E402
from laml_gb300.autograd import log_likelihood  # noqa: E402
from oracle import pmm_oracle as O  # noqa: E402


def _setup(compat, n=64, K=20, seed=21):
    w = synth.pmm_workload(n, K, 4, 20, 0.3, 0.05, 0.1, seed=seed)
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=compat, clamp=False)
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    prob = O.Problem(tr, O.recode([w.rows[c] for c in w.leaf_order], w.Q, compat=compat), compat)
    return w, b, prob


def _grad(b, d, nu, phi, recompute=False):
    dt = torch.tensor(d, dtype=torch.float64, device="cuda", requires_grad=True)
    nt = torch.tensor([nu], dtype=torch.float64, device="cuda", requires_grad=True)
    pt = torch.tensor([phi], dtype=torch.float64, device="cuda", requires_grad=True)
    llh = log_likelihood(dt, nt, pt, b, recompute=recompute)
    llh.sum().backward()
    return float(llh[0]), dt.grad.cpu().numpy(), float(nt.grad[0]), float(pt.grad[0])


@pytest.mark.parametrize("compat", [True, False])
def test_gradient_matches_finite_differences(compat):
    w, b, prob = _setup(compat)
    d = prob.tree.branch_lengths.copy()
    nu, phi = 0.07, 0.12
    llh, gd, gnu, gphi = _grad(b, d, nu, phi)
    ref = O.log_likelihood(prob, d, nu, phi)[0]
    assert llh == pytest.approx(ref, rel=1e-6)
    h = 1e-4
    rng = np.random.default_rng(0)
    for v in rng.choice(len(d), 12, replace=False):
        dp, dm = d.copy(), d.copy()
        dp[v] += h
        dm[v] -= h
        fd = (O.log_likelihood(prob, dp, nu, phi)[0] - O.log_likelihood(prob, dm, nu, phi)[0]) / (2 * h)
        assert gd[v] == pytest.approx(fd, rel=1e-3, abs=1e-3), v
    fd_nu = (O.log_likelihood(prob, d, nu + h, phi)[0] - O.log_likelihood(prob, d, nu - h, phi)[0]) / (2 * h)
    fd_phi = (O.log_likelihood(prob, d, nu, phi + h)[0] - O.log_likelihood(prob, d, nu, phi - h)[0]) / (2 * h)
    assert gnu == pytest.approx(fd_nu, rel=1e-3, abs=1e-3)
    assert gphi == pytest.approx(fd_phi, rel=1e-3, abs=1e-3)


def test_gradient_equals_reference_objective_gradient():
    """The gradient of M_step_loss_fn (laml.py:62-78) in (d, nu, phi) at the
    current parameters, with oracle counts whose root row is the progenitor's."""
    w, b, prob = _setup(True)
    d = prob.tree.branch_lengths.copy()
    nu, phi = 0.07, 0.12
    _, gd, gnu, gphi = _grad(b, d, nu, phi)
    root = prob.tree.root
    es_true = O.e_step(prob, d, nu, phi)
    # the root row from the progenitor in state 0 (compat semantics otherwise)
    cnt = es_true.counts.copy()
    t = O.branch_terms(d, nu, O.EPS)
    iv = es_true.inside[root]
    L = es_true.llh_site
    cnt[root, 0] = np.exp(iv[:, 0] + t[3][root] - L).sum()
    cnt[root, 1] = np.exp(O.lse(iv[:, 1:-1] + t[0][root] + prob.logq + t[2][root], 1) - L).sum()
    cnt[root, 2] = np.exp(iv[:, -1] + t[1][root] - L).sum()
    cnt[root, 3:] = 0.0
    e = cnt
    em = np.expm1(d)
    g_ref = -e[:, 0] * (1 + nu) + e[:, 1] * (1 / em - nu) + (e[:, 2] + e[:, 4]) * nu / np.expm1(nu * d) - e[:, 3] * nu
    np.testing.assert_allclose(gd, g_ref, rtol=1e-3, atol=1e-3)
    gnu_ref = np.sum(-(e[:, 0] + e[:, 1] + e[:, 3]) * d + (e[:, 2] + e[:, 4]) * d / np.expm1(nu * d))
    assert gnu == pytest.approx(gnu_ref, rel=1e-3, abs=1e-3)
    n = prob.tree.num_leaves
    M = float(np.sum(prob.enc.chars == O.MISSING))
    R = prob.enc.chars.size - M
    miss = prob.enc.chars == O.MISSING
    p1 = np.exp(es_true.post1[:n])
    gphi_ref = -(R - p1[~miss].sum()) / (1 - phi) + (M - p1[miss].sum()) / phi
    assert gphi == pytest.approx(gphi_ref, rel=1e-3, abs=1e-3)


def test_recompute_equals_stored():
    w, b, prob = _setup(True, seed=22)
    d = prob.tree.branch_lengths.copy()
    a = _grad(b, d, 0.05, 0.1, recompute=False)
    c = _grad(b, d, 0.05, 0.1, recompute=True)
    assert a[0] == c[0]
    np.testing.assert_array_equal(a[1], c[1])
    assert a[2] == c[2] and a[3] == c[3]
