"""The C restatement (oracle/pmm_oracle.c) equals the NumPy oracle."""
import numpy as np

from laml_gb300 import synth
from oracle import cpu_port
from oracle import pmm_oracle as O


def test_c_port_matches_numpy_oracle():
    w = synth.pmm_workload(40, 12, 3, 12, 0.5, 0.1, 0.15, seed=3, n_trees=3)
    llh, nu, phi, ds, _ = cpu_port.em(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5, iters=3)
    for i in range(3):
        tr = O.parse_tree(w.newicks[i], w.leaf_order)
        enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, True)
        r = O.em_compat(O.Problem(tr, enc, True), tr.branch_lengths, 0.5, 0.5, max_iters=3,
                        stop=-1)
        assert abs(llh[i] / r.llh - 1) < 1e-12
        assert abs(nu[i] / r.nu - 1) < 1e-10
        assert abs(phi[i] / r.phi - 1) < 1e-12
        np.testing.assert_allclose(ds[i], r.d, rtol=1e-10)


def test_zero_count_branch_keeps_its_length():
    """A branch whose expected counts are all zero (fast_em's root row on a
    large tree) has a zero M-step gradient; L-BFGS leaves it unchanged."""
    rng = np.random.default_rng(0)
    cnt = rng.uniform(0.1, 2.0, (5, 6))
    cnt[2] = 0.0
    d0 = np.array([0.1, 0.2, 0.37, 0.4, 0.5])
    d, nu, phi = O.mstep_compat(cnt, 1.0, 10.0, 5.0, d0, 0.3, 0.2, np.ones(5, bool), False,
                                False)
    assert d[2] == d0[2]
    assert np.all(d[[0, 1, 3, 4]] != d0[[0, 1, 3, 4]])


def test_c_port_large_tree_root_row():
    """1500 leaves, 8 sites: the compat root row is all zero; both oracles
    keep the root branch and the EM climbs."""
    w = synth.pmm_workload(1500, 8, 3, 10, 0.5, 0.1, 0.15, seed=31)
    llh, nu, phi, ds, _ = cpu_port.em(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5, iters=2)
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, True)
    r = O.em_compat(O.Problem(tr, enc, True), tr.branch_lengths, 0.5, 0.5, max_iters=2, stop=-1)
    assert r.trace[1] > r.trace[0] and r.trace[2] > r.trace[1]
    assert abs(llh[0] / r.llh - 1) < 1e-12
    np.testing.assert_allclose(ds[0], r.d, rtol=1e-10)


def test_c_port_loglik_forms_match_numpy_oracle():
    """The whole-tree (ora_loglik) and per-site (ora_site_loglik) forms of the
    C restatement give the NumPy oracle's per-site and total log-likelihood."""
    w = synth.pmm_workload(60, 17, 3, 14, 0.5, 0.1, 0.15, seed=7, n_trees=3)
    enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, True)
    ll = cpu_port.loglik(w.newicks, w.rows, w.Q, w.leaf_order, 0.13, 0.21)
    for i in range(3):
        tr = O.parse_tree(w.newicks[i], w.leaf_order)
        d = tr.branch_lengths * (1.0 + 0.1 * i)
        ref, ref_site = O.log_likelihood(O.Problem(tr, enc, True), d, 0.13, 0.21)
        site = cpu_port.site_loglik(w.newicks[i], w.rows, w.Q, w.leaf_order, 0.13, 0.21, d=d,
                                    enc=enc)
        np.testing.assert_allclose(site, ref_site, rtol=1e-12)
        assert abs(site.sum() / ref - 1) < 1e-12
        if i == 0:
            assert abs(ll[0] / O.log_likelihood(O.Problem(tr, enc, True), tr.branch_lengths,
                                                0.13, 0.21)[0] - 1) < 1e-12
