"""The oracle's restatement of fastEM's own M-step (100 L-BFGS steps with
the zoom line search, FP32; fast_em/laml.py:49-110): its gradient against
central differences of its loss (h = 1e-2), its descent, its masks, and its end point
against the stationary-point solve of the same objective."""
import numpy as np
import pytest

from laml_gb300 import synth
from oracle import pmm_oracle as O


def _counts(seed=5):
    w = synth.pmm_workload(40, 12, 3, 10, 0.5, 0.1, 0.15, seed=seed)
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    prob = O.Problem(tr, O.recode([w.rows[c] for c in w.leaf_order], w.Q, True), True)
    es = O.e_step(prob, tr.branch_lengths, 0.3, 0.2)
    M = float(np.sum(prob.enc.chars == O.MISSING))
    return tr, es, M, prob.enc.chars.size - M


def test_loss_gradient_matches_differences():
    tr, es, M, R = _counts()
    N = len(tr.parent)
    x = O.lbfgs_start(tr.branch_lengths, 0.3, 0.2).astype(np.float64)
    ones = np.ones(N)
    f0, g = O.mstep_loss_grad(x, es.counts, es.leaf_resp.sum(), R, M, ones, [1, 1])
    rng = np.random.default_rng(0)
    for i in list(rng.choice(N, 6, replace=False)) + [N, N + 1]:
        h = 1e-2
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        fp = O.mstep_loss_grad(xp, es.counts, es.leaf_resp.sum(), R, M, ones, [1, 1])[0]
        fm = O.mstep_loss_grad(xm, es.counts, es.leaf_resp.sum(), R, M, ones, [1, 1])[0]
        fd = (float(fp) - float(fm)) / (2 * h)
        assert g[i] == pytest.approx(fd, rel=2e-2, abs=2e-2 * max(1.0, abs(float(f0)) * 1e-4))


def test_lbfgs_mstep_descends_respects_masks_and_reaches_the_stationary_point():
    tr, es, M, R = _counts()
    N = len(tr.parent)
    lr = float(es.leaf_resp.sum())
    mask = np.ones(N, bool)
    mask[3] = False
    x0 = O.lbfgs_start(tr.branch_lengths, 0.3, 0.2)
    x = O.mstep_compat_lbfgs(es.counts, lr, R, M, x0, mask, False, True)
    f0 = O.mstep_loss_grad(x0, es.counts, lr, R, M, mask, [1, 0])[0]
    f1 = O.mstep_loss_grad(x, es.counts, lr, R, M, mask, [1, 0])[0]
    assert f1 < f0
    assert x[3] == x0[3] and x[N + 1] == x0[N + 1]   # masked: unchanged
    d, nu, phi = O.mstep_compat(es.counts, lr, R, M, tr.branch_lengths, 0.3, 0.2, mask, False,
                                True)
    fs = -O.mstep_objective_compat(es.counts, lr, R, M, d, nu, phi)
    assert float(f1) == pytest.approx(fs, rel=1e-5)
