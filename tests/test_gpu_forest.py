"""Several trees in one EM on the device (the trees joined under
zero-length fixed branches, laml_gb300/forest.py) against the oracle's
restatement of EM_solver with a list of trees (oracle em_exact_forest:
per-tree E-steps, one M-step, root rows for ultra_constr).

* 5 fixed EM iterations of 2 and 3 trees, with and without the ultrametric
  equalities: the summed log-likelihood to 1e-6 relative, nu and phi to
  1e-3, branch lengths to 1e-3 relative (FP32 E-step counts against FP64);
  under ultra_constr every leaf of every tree at one height (1e-9).
* the EM_solver drop-in's optimize() with two trees reaches the oracle's
  fixed point from the same start (1e-6 relative in log-likelihood)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from laml_gb300 import synth  # noqa: E402
from laml_gb300.encoding import char_matrix, encode_dataset, encode_newick  # noqa: E402
from laml_gb300.engine import DeviceBatch  # noqa: E402
from laml_gb300.forest import join_forest  # noqa: E402
from oracle import pmm_oracle as O  # noqa: E402


def _case(k):
    return synth.pmm_workload(60, 20, 3, 10, 0.5, 0.1, 0.15, seed=40 + k, n_trees=k)


@pytest.mark.parametrize("k", [2, 3])
@pytest.mark.parametrize("ultra", [False, True])
def test_forest_em_matches_oracle(k, ultra):
    w = _case(k)
    trees = [encode_newick(nw, w.leaf_order) for nw in w.newicks]
    rng = np.random.default_rng(k)
    ds = [rng.uniform(0.05, 0.6, t.num_nodes) for t in trees]
    joined, maps, joins = join_forest(trees)
    rows = [w.rows[c] for _ in range(k) for c in w.leaf_order]
    dset = encode_dataset(char_matrix(rows, exact=True), w.Q, compat=False)
    dj = np.zeros(joined.num_nodes)
    mj = np.ones(joined.num_nodes, bool)
    mj[joins] = False
    for m, d in zip(maps, ds):
        dj[m] = d
    b = DeviceBatch([dset], [joined], [0], [dj], [0.3], [0.2], compat=False, mask=[mj],
                    ultrametric=ultra)
    r = b.run_em(max_iters=5, rel_tol=-1.0, chunk=1)[0]
    b.check_device_error()
    enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, compat=False)
    probs = [O.Problem(O.parse_tree(nw, w.leaf_order), enc, False) for nw in w.newicks]
    ref = O.em_exact_forest(probs, ds, 0.3, 0.2, max_iters=5, stop=-1.0, ultra=ultra)
    assert r.iterations == 5
    assert r.llh == pytest.approx(ref.llh, rel=1e-6)
    assert r.nu == pytest.approx(ref.nu, rel=1e-3, abs=1e-6)
    assert r.phi == pytest.approx(ref.phi, rel=1e-3, abs=1e-6)
    for t in range(k):
        np.testing.assert_allclose(r.branch_lengths[maps[t]], ref.d[t], rtol=1e-3, atol=1e-6)
    if ultra:
        h = []
        for t, tr in enumerate(trees):
            for leaf in range(tr.num_leaves):
                x, s = leaf, 0.0
                while x >= 0:
                    s += r.branch_lengths[maps[t][x]]
                    x = tr.parent[x]
                h.append(s)
        assert np.ptp(h) <= 1e-9 * max(h)


def test_em_solver_dropin_two_trees():
    from laml_gb300.fastEM_solver import EM_solver
    w = _case(2)
    s = EM_solver(w.newicks, {"charMtrx": w.rows, "ordered_leaf_labels": [w.leaf_order] * 2},
                  {"Q": w.Q})
    nllh, status = s.optimize(initials=1, random_seeds=[7], verbose=-1)
    assert status == "optimal"
    # the oracle from the drop-in's own start (EM_solver's initial point)
    import random
    enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, compat=False)
    probs = [O.Problem(O.parse_tree(nw, w.leaf_order), enc, False) for nw in w.newicks]
    rs = random.Random(7)
    post = [O.treeswift_postorder_ids(p.tree) for p in probs]
    x = [rs.random() * (O.DMAX / 2 - 2 * O.DMIN) + 2 * O.DMIN for _ in range(sum(map(len, post)))]
    nu, phi = rs.random() * 0.99, rs.random() * 0.99
    ds, k = [], 0
    for p, po in zip(probs, post):
        d = np.empty(len(p.tree.parent))
        for u in po:
            L = p.tree.branch_lengths[u]
            d[u] = max(2 * O.DMIN, L)
            k += 1
        ds.append(d)
    ref = O.em_exact_forest(probs, ds, nu, phi)
    assert -nllh == pytest.approx(ref.llh, rel=1e-6)
    assert sum(len(t) for t in s.get_tree_newick()) > 0
