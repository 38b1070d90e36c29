"""fastEM's own M-step on the device (LAML_MSTEP_LBFGS: 100 FP32 L-BFGS
steps with the zoom line search, fast_em/laml.py:49-110) against the
oracle's restatement (pmm_oracle.mstep_compat_lbfgs) on the device's own
expected counts, and an EM with it against the oracle's EM with the same
M-step.  100 L-BFGS steps do not reach the stationary point of a 79-branch
objective, and two FP32 runs whose summation orders differ follow apart in
its flat directions (short branches: up to 30% apart at 1e-4): the objective
reached agrees to 1e-5 relative, nu and phi to 1e-2, the log-likelihood of 5
EM iterations to 3e-5 relative (measured 1.1e-5).  The 4-leaf NNI searches
with it are in test_gpu_topology.py."""
import random

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from laml_gb300 import problem as PB  # noqa: E402
from laml_gb300 import synth  # noqa: E402
from oracle import pmm_oracle as O  # noqa: E402


def _case():
    return synth.pmm_workload(40, 12, 3, 10, 0.5, 0.1, 0.15, seed=5)


def test_lbfgs_mstep_matches_oracle_on_device_counts():
    w = _case()
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, nu=0.3, phi=0.2)
    b.lbfgs = True
    b.e_step()
    b.mstep()
    torch.cuda.synchronize()
    b.check_device_error()
    r = b.results()[0]
    N_ = b.trees[0].num_nodes
    cnt = b.work["nd_cnt"].cpu().numpy().reshape(-1, 6)[:N_]
    cp = b.work["cnt_part"].cpu().numpy()
    ng = b.datasets[0].n_groups
    lr = float(cp[:N_ * ng * 8].reshape(N_, ng, 8)[:, :, 6:8].astype(np.float64).sum())
    ds = b.datasets[0]
    M = float(ds.n_missing)
    R = float(N_ // 2 + 1) * ds.n_sites - M
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    x0 = O.lbfgs_start(np.maximum(tr.branch_lengths, 1e-6), 0.3, 0.2)
    mask = np.ones(N_, bool)
    x = O.mstep_compat_lbfgs(cnt, lr, R, M, x0, mask, False, False)
    d, nu, phi = O.lbfgs_params(x)
    f_or = O.mstep_loss_grad(x, cnt, lr, R, M, mask, [1, 1])[0]
    xg = O.lbfgs_start(r.branch_lengths, r.nu, r.phi)
    xg[:N_] = np.log(r.branch_lengths)
    f_gpu = O.mstep_loss_grad(xg, cnt, lr, R, M, mask, [1, 1])[0]
    assert float(f_gpu) == pytest.approx(float(f_or), rel=1e-5)
    f0 = O.mstep_loss_grad(x0, cnt, lr, R, M, mask, [1, 1])[0]
    assert float(f_gpu) < float(f0)
    assert r.nu == pytest.approx(nu, rel=1e-2, abs=1e-6)
    assert r.phi == pytest.approx(phi, rel=1e-2, abs=1e-6)


def test_em_with_lbfgs_mstep_matches_oracle():
    w = _case()
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, nu=0.5, phi=0.5)
    b.lbfgs = True
    r = b.run_em(max_iters=5, rel_tol=-1.0, chunk=1)[0]
    b.check_device_error()
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    prob = O.Problem(tr, O.recode([w.rows[c] for c in w.leaf_order], w.Q, True), True)
    ref = O.em_compat(prob, tr.branch_lengths, 0.5, 0.5, max_iters=5, stop=-1.0, mstep="lbfgs")
    assert r.iterations == 5
    assert r.llh == pytest.approx(ref.llh, rel=3e-5)
    assert r.nu == pytest.approx(ref.nu, rel=1e-2, abs=1e-6)
