"""GPU ultrametric M-step (LAML_MSTEP_ULTRAMETRIC) against the oracle.

EM_solver.Mstep with ultra_constr_cache (laml_libs/EM_solver.py:53-89,
349-366).  Tolerances:

* the device solve and the oracle's (LP start + dense null-space barrier) on
  the same normalised counts (the device's nd_cnt): branch lengths 3e-6
  relative (+1e-7 absolute, for branches at a bound), objective 1e-9
  relative (the device's transcendental cores are FP32);
* a whole M-step with the oracle's FP64 E-step counts (the device's counts
  are FP32 sums): branch lengths 1e-3 relative (+1e-6), nu and phi 1e-4;
* every solution is ultrametric: root-to-leaf paths below the root equal to
  1e-9 relative, every branch inside [dmin, dmax];
* the exact EM through the drop-in solver: each of the 15 rooted four-leaf
  topologies of unit_tests_TopoSearch.py test_10 at the oracle's fixed point
  (1e-6 relative), the best at that test's pre-computed optimum (places=4).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from laml_gb300 import _native as N  # noqa: E402
from laml_gb300 import problem as PB  # noqa: E402
from laml_gb300 import synth  # noqa: E402
from oracle import pmm_oracle as O  # noqa: E402
from tests.helpers import rooted_topologies, ultrametric_cases  # noqa: E402


def _paths(parent, n_leaves, d):
    out = np.zeros(n_leaves)
    for leaf in range(n_leaves):
        x, s = leaf, 0.0
        while parent[x] >= 0:
            s += d[x]
            x = parent[x]
        out[leaf] = s
    return out


def _objective(S, nu, d, mask):
    S0, S1, S2, S3, S4 = (S[:, i] for i in range(5))
    a = (nu + 1) * S0 + nu * S1 + nu * S3
    v = -a * d + S1 * O._log1mexp(d)
    if nu > O.EPS_NU:
        v = v + (S2 + S4) * O._log1mexp(nu * d)
    return float(np.sum(v[mask]))


def _start(tree_parent, rng, lo=0.05, hi=0.8):
    return rng.uniform(lo, hi, size=len(tree_parent))


def _ultrametric_lengths(tr, rng):
    """Branch lengths of an ultrametric tree (heights grow by U(0.05, 0.3)
    above the taller child): fixing any of them keeps the problem feasible."""
    P = np.zeros(len(tr.parent))
    for u in O.treeswift_postorder_ids(tr):
        if tr.children[u]:
            P[u] = max(P[c] for c in tr.children[u]) + rng.uniform(0.05, 0.3)
    d = np.full(len(tr.parent), 0.2)
    for x in range(len(tr.parent)):
        if tr.parent[x] >= 0:
            d[x] = P[tr.parent[x]] - P[x]
    return d


CASES = [  # leaves, sites, seed, nu, fraction of fixed branches
    (12, 10, 1, 0.1, 0.0),
    (60, 20, 2, 0.2, 0.0),
    (200, 30, 3, 0.05, 0.0),
    (80, 16, 4, 1e-6, 0.0),    # nu below eps_nu: no silencing terms
    (90, 16, 5, 0.1, 0.15),    # fixed branches inside the equalities
]


@pytest.mark.parametrize("n,K,seed,nu,fixed", CASES)
def test_ultrametric_solve_matches_oracle_on_device_counts(n, K, seed, nu, fixed):
    w = synth.pmm_workload(n, K, 3, 12, 0.5, 0.1, 0.15, seed=seed)
    rng = np.random.default_rng(seed)
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    N_ = len(tr.parent)
    d0 = _start(tr.parent, rng)
    mask = rng.random(N_) >= fixed
    if fixed > 0:   # fixed branches at the lengths of an ultrametric tree
        d0 = np.where(mask, d0, _ultrametric_lengths(tr, rng))
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=False, nu=nu, phi=0.15,
                      d=[d0], mask=[mask], clamp=False, ultrametric=True, fix_nu=True,
                      fix_phi=True)
    b.e_step()
    b.mstep()
    torch.cuda.synchronize()
    r = b.results()[0]
    assert r.status == N.TREE_ACTIVE
    S = b.work["nd_cnt"].cpu().numpy().reshape(-1, 6)[:N_, :5]
    od, ok = O.ultrametric_d(S, nu, d0, mask, tr)
    assert ok
    np.testing.assert_allclose(r.branch_lengths, od, rtol=3e-6, atol=1e-7)
    fd, fo = _objective(S, nu, r.branch_lengths, mask), _objective(S, nu, od, mask)
    assert fd >= fo - 1e-9 * abs(fo)
    assert np.all(r.branch_lengths[mask] >= O.DMIN - 1e-12)
    assert np.all(r.branch_lengths[mask] <= O.DMAX + 1e-12)
    assert np.array_equal(r.branch_lengths[~mask], d0[~mask])
    p = _paths(tr.parent, tr.num_leaves, r.branch_lengths)
    assert np.ptp(p) <= 1e-9 * np.max(p)


@pytest.mark.parametrize("n,K,seed,nu,fixed", CASES[:3])
def test_ultrametric_mstep_matches_oracle_mstep(n, K, seed, nu, fixed):
    w = synth.pmm_workload(n, K, 3, 12, 0.5, 0.1, 0.15, seed=seed)
    rng = np.random.default_rng(seed)
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    d0 = _start(tr.parent, rng)
    phi = 0.15
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=False, nu=nu, phi=phi,
                      d=[d0], clamp=False, ultrametric=True)
    b.e_step()
    b.mstep()
    torch.cuda.synchronize()
    r = b.results()[0]
    enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, compat=False)
    prob = O.Problem(tr, enc, False)
    es = O.e_step(prob, d0, nu, phi)
    lstat, R = O.exact_leaf_stats(prob, es)
    od, onu, ophi, ok = O.mstep_exact(es.counts, lstat, R, d0, nu, phi,
                                      np.ones(len(d0), bool), enc.chars.shape[1],
                                      tr.num_leaves, ultra_tree=tr)
    assert ok
    np.testing.assert_allclose(r.branch_lengths, od, rtol=1e-3, atol=1e-6)
    assert r.nu == pytest.approx(onu, rel=1e-4, abs=1e-8)
    assert r.phi == pytest.approx(ophi, rel=1e-4, abs=1e-8)


def test_ultrametric_em_paths_agree():
    """The persistent kernel and the per-level graph run the same M-step."""
    w = synth.pmm_workload(70, 14, 3, 12, 0.5, 0.1, 0.15, seed=8, n_trees=3)
    rng = np.random.default_rng(8)
    ds = [_start(O.parse_tree(nw, w.leaf_order).parent, rng) for nw in w.newicks]
    res = {}
    for path in ("graph", "persistent", "levels"):
        b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=False, nu=0.3,
                          phi=0.2, d=ds, clamp=False, ultrametric=True)
        res[path] = b.run_em(max_iters=6, rel_tol=-1.0, chunk=2, path=path)
    for t in range(3):
        for path in ("persistent", "levels"):
            assert res[path][t].llh == res["graph"][t].llh
            np.testing.assert_array_equal(res[path][t].branch_lengths,
                                          res["graph"][t].branch_lengths)
        tr = O.parse_tree(w.newicks[t], w.leaf_order)
        p = _paths(tr.parent, tr.num_leaves, res["graph"][t].branch_lengths)
        assert np.ptp(p) <= 1e-9 * np.max(p)


def test_ultrametric_cluster_equals_block():
    """A tree above 16384 nodes: the cluster M-step (8 blocks, distributed
    shared memory reductions) against one block on the same counts."""
    w = synth.pmm_workload(9000, 8, 3, 10, 0.5, 0.1, 0.15, seed=9)
    rng = np.random.default_rng(9)
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    d0 = _start(tr.parent, rng)
    out = []
    for force_block in (False, True):
        b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=False, nu=0.1,
                          phi=0.15, d=[d0], clamp=False, ultrametric=True)
        if force_block:
            b.b.max_tree_nodes = 1   # k_mstep then takes every tree on one block
        b.e_step()
        b.mstep()
        torch.cuda.synchronize()
        out.append(b.results()[0])
    assert out[0].status == out[1].status == N.TREE_ACTIVE
    np.testing.assert_allclose(out[0].branch_lengths, out[1].branch_lengths, rtol=1e-7,
                               atol=1e-9)
    p = _paths(tr.parent, tr.num_leaves, out[0].branch_lengths)
    assert np.ptp(p) <= 1e-9 * np.max(p)
    assert np.all(out[0].branch_lengths >= O.DMIN - 1e-12)


def test_ultrametric_infeasible_keeps_parameters():
    msa = {"a": [1, 0, 1], "b": [1, 1, 0], "c": [0, 1, 1]}
    Q = [{1: 1.0}] * 3
    leaves = ["a", "b", "c"]
    # a fixed at 20 > dmax: its sibling b would need the same length
    nw = "((a:20,b:2):1,c:1):0.5;"
    trees = PB.encode_trees([nw], leaves)
    mask = np.ones(5, bool)
    mask[0] = False
    b = PB.make_batch([nw], msa, Q, leaves, compat=False, nu=0.1, phi=0.1, mask=[mask],
                      clamp=False, ultrametric=True, trees=trees)
    llh0 = float(b.log_likelihood()[0])
    r = b.run_em(max_iters=50)[0]
    assert r.status == N.TREE_INFEASIBLE
    np.testing.assert_array_equal(r.branch_lengths, trees[0].branch_length)
    assert (r.nu, r.phi) == (0.1, 0.1)
    assert r.llh == pytest.approx(llh0, rel=1e-12)
    # both cherry branches fixed and unequal: the reference drops that row
    nw = "((a:1,b:2):1,c:1):0.5;"
    mask[1] = False
    b = PB.make_batch([nw], msa, Q, leaves, compat=False, nu=0.1, phi=0.1, mask=[mask],
                      clamp=False, ultrametric=True)
    r = b.run_em(max_iters=50)[0]
    assert r.status in (N.TREE_CONVERGED, N.TREE_MAXITER)


def test_dropin_optimize_ultra_bruteforce():
    """fastEM_solver.optimize(ultra_constr=True) (ML_solver.optimize ->
    EM_solver.optimize_one with the ultrametric M-step) on every rooted
    topology of the four-leaf test_10 case."""
    from laml_gb300.fastEM_solver import fastEM_solver
    (case,) = ultrametric_cases()
    leaves = case["leaves"]
    best = np.inf
    for top in rooted_topologies(leaves):
        nw = top + ";"
        s = fastEM_solver([nw], {"charMtrx": case["msa"], "ordered_leaf_labels": [leaves]},
                          {"Q": case["Q"]}, {"nu": 0.0, "phi": 0.0})
        nllh, status = s.optimize(initials=1, verbose=-1, random_seeds=1, ultra_constr=True)
        assert status == "optimal"
        tr = O.parse_tree(nw, leaves)
        enc = O.recode([case["msa"][c] for c in leaves], case["Q"], compat=False)
        prob = O.Problem(tr, enc, False)
        post = O.treeswift_postorder_ids(tr)
        x, nu, phi = O.exact_initials(tr, [None] * len(post), 1)
        d = np.empty(len(tr.parent))
        for i, u in enumerate(post):
            d[u] = x[i]
        ref = O.em_exact(prob, d, nu, phi, ultra=True)
        assert nllh == pytest.approx(-ref.llh, rel=1e-6)
        best = min(best, nllh)
    assert round(best - case["nllh_bf"], 4) == 0


def test_topology_search_ultrametric_em_solver():
    """unit_tests_TopoSearch.py test_9: NNI search with EM_solver and
    ultra_constr from ((a,b),(c,d)) reaches the brute-force ultrametric
    optimum (places=4)."""
    from copy import deepcopy
    from laml_gb300.fastEM_solver import EM_solver
    from laml_gb300.topology_search import DEFAULT_STRATEGY, Topology_search
    (case,) = ultrametric_cases()
    data = {"charMtrx": case["msa"]}
    prior = {"Q": case["Q"]}
    search = Topology_search(["((a,b),(c,d));"], EM_solver, data=data, prior=prior,
                             params={"phi": 0, "nu": 0})
    strategy = deepcopy(DEFAULT_STRATEGY)
    strategy["ultra_constr"] = True
    _, max_score, _ = search.search(maxiter=200, verbose=False, strategy=strategy, nreps=1)
    assert round(-max_score - case["nllh_bf"], 4) == 0


@pytest.mark.parametrize("mode", ["barrier", "pd_short"])
@pytest.mark.parametrize("n,K,seed,nu,fixed", [CASES[1], CASES[4]])
def test_ultrametric_barrier_only_matches_primal_dual(n, K, seed, nu, fixed, mode):
    """The primal-dual method's fallback solves the same M-step, against the
    oracle on the device's counts and against the primal-dual solution:
    LAML_MSTEP_ULTRA_BARRIER (the log-barrier method alone) and
    LAML_MSTEP_ULTRA_PD_SHORT (3 primal-dual iterations, then the barrier
    method from the near-boundary point they reach)."""
    w = synth.pmm_workload(n, K, 3, 12, 0.5, 0.1, 0.15, seed=seed)
    rng = np.random.default_rng(seed)
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    N_ = len(tr.parent)
    d0 = _start(tr.parent, rng)
    mask = rng.random(N_) >= fixed
    if fixed > 0:
        d0 = np.where(mask, d0, _ultrametric_lengths(tr, rng))
    out = []
    for barrier in (False, True):
        b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=False, nu=nu,
                          phi=0.15, d=[d0], mask=[mask], clamp=False, ultrametric=True,
                          fix_nu=True, fix_phi=True)
        b.ultra_barrier = barrier and mode == "barrier"
        b.ultra_pd_short = barrier and mode == "pd_short"
        b.e_step()
        b.mstep()
        torch.cuda.synchronize()
        out.append((b.results()[0], b.work["nd_cnt"].cpu().numpy().reshape(-1, 6)[:N_, :5]))
    (rp, Sp), (rb, Sb) = out
    np.testing.assert_array_equal(Sp, Sb)   # the same E-step
    od, ok = O.ultrametric_d(Sb, nu, d0, mask, tr)
    assert ok
    np.testing.assert_allclose(rb.branch_lengths, od, rtol=3e-6, atol=1e-7)
    np.testing.assert_allclose(rb.branch_lengths, rp.branch_lengths, rtol=3e-6, atol=1e-7)
    p = _paths(tr.parent, tr.num_leaves, rb.branch_lengths)
    assert np.ptp(p) <= 1e-9 * np.max(p)
