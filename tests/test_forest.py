"""Several trees in one EM (laml_gb300/forest.py): the oracle's restatement
of EM_solver with a list of trees (per-tree E-steps, one M-step over all of
them, EM_solver.py:307-512, and for ultra_constr the root rows of
EM_solver.py:81-84) against the same EM on the trees joined under
zero-length fixed branches -- the form the device runs -- in FP64, with and
without the ultrametric equalities; and the host join itself."""
import numpy as np
import pytest

from laml_gb300 import synth
from laml_gb300.encoding import encode_newick
from laml_gb300.forest import join_forest
from oracle import pmm_oracle as O


def _forest(k=2, n=14, K=9, seed=3):
    w = synth.pmm_workload(n, K, 3, 8, 0.5, 0.1, 0.15, seed=seed, n_trees=k)
    return w


def _joined_problem(w, k):
    """The k trees under a caterpillar of joining nodes J0.. (branch 0), each
    tree's leaves renamed apart, as one oracle problem."""
    parts = []
    rows = {}
    for t in range(k):
        s = w.newicks[t].strip().rstrip(";")
        for c in w.leaf_order:
            s = s.replace(c + ":", f"{c}#{t}:")
            rows[f"{c}#{t}"] = w.rows[c]
        parts.append(s)
    nw = parts[-1]
    for j in range(k - 2, -1, -1):
        nw = f"({parts[j]},{nw})J{j}:0.0"
    nw += ";"
    order = [f"{c}#{t}" for t in range(k) for c in w.leaf_order]
    tr = O.parse_tree(nw, order)
    enc = O.recode([rows[c] for c in order], w.Q, compat=False)
    return O.Problem(tr, enc, False), tr


def _per_tree(w, k):
    enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, compat=False)
    return [O.Problem(O.parse_tree(w.newicks[t], w.leaf_order), enc, False) for t in range(k)]


@pytest.mark.parametrize("k", [2, 3])
@pytest.mark.parametrize("ultra", [False, True])
def test_forest_em_equals_joined_tree_em(k, ultra):
    w = _forest(k=k)
    probs = _per_tree(w, k)
    rng = np.random.default_rng(k)
    ds = [rng.uniform(0.05, 0.6, len(p.tree.parent)) for p in probs]
    ref = O.em_exact_forest(probs, ds, 0.3, 0.2, max_iters=4, stop=-1.0, ultra=ultra)
    jp, jt = _joined_problem(w, k)
    # joined ids of each tree's nodes: by label (leaves renamed, internal
    # nodes by their order within the tree)
    lab = {l: i for i, l in enumerate(jt.labels)}
    dj = np.zeros(len(jt.parent))
    mask = np.ones(len(jt.parent), bool)
    for j in range(k - 1):
        mask[lab[f"J{j}"]] = False
    maps = []
    for t, p in enumerate(probs):
        m = np.empty(len(p.tree.parent), np.int64)
        for u in range(p.tree.num_leaves):
            m[u] = lab[f"{p.tree.labels[u]}#{t}"]
        maps.append(m)
    # internal nodes: match by the set of leaves below
    def clades(tr, leafname):
        out = {}
        for u in O.treeswift_postorder_ids(tr):
            ch = tr.children[u]
            out[u] = frozenset([leafname(u)]) if not ch else frozenset().union(*[out[c] for c in ch])
        return out
    jc = clades(jt, lambda u: jt.labels[u])
    inv = {v: u for u, v in jc.items()}
    for t, p in enumerate(probs):
        pc = clades(p.tree, lambda u: f"{p.tree.labels[u]}#{t}")
        for u in range(p.tree.num_leaves, len(p.tree.parent)):
            maps[t][u] = inv[pc[u]]
        dj[maps[t]] = ds[t]
    got = O.em_exact(jp, dj, 0.3, 0.2, branch_mask=mask, max_iters=4, stop=-1.0, ultra=ultra)
    assert got.llh == pytest.approx(ref.llh, rel=1e-9)
    assert got.nu == pytest.approx(ref.nu, rel=1e-7, abs=1e-12)
    assert got.phi == pytest.approx(ref.phi, rel=1e-7, abs=1e-12)
    for t in range(k):
        np.testing.assert_allclose(got.d[maps[t]], ref.d[t], rtol=1e-6, atol=1e-9)
    if ultra:   # every leaf of every tree at one height above the joined root
        h = []
        for t in range(k):
            tr = probs[t].tree
            for leaf in range(tr.num_leaves):
                x, s = leaf, 0.0
                while x >= 0:
                    s += ref.d[t][x]
                    x = tr.parent[x]
                h.append(s)
        assert np.ptp(h) <= 1e-8 * max(h)


def test_join_forest_structure():
    w = _forest(k=3)
    trees = [encode_newick(nw, w.leaf_order) for nw in w.newicks]
    j, maps, joins = join_forest(trees)
    assert j.num_nodes == sum(t.num_nodes for t in trees) + 2
    assert j.num_leaves == 3 * trees[0].num_leaves
    assert j.root == joins[0] and len(joins) == 2
    for t, m in zip(trees, maps):
        np.testing.assert_array_equal(j.branch_length[m], t.branch_length)
        for u in range(t.num_nodes):   # parent structure carried over
            if t.parent[u] >= 0:
                assert j.parent[m[u]] == m[t.parent[u]]
            else:
                assert j.parent[m[u]] in joins
        assert np.all(m[:t.num_leaves] < j.num_leaves) and np.all(m[t.num_leaves:] >= j.num_leaves)
    assert np.all(j.branch_length[joins] == 0.0)
    assert np.all(j.parent[np.arange(j.num_nodes)[j.parent >= 0]] < j.num_nodes)
    # parents precede children among internal nodes
    inner = np.arange(j.num_leaves, j.num_nodes)
    assert np.all(j.parent[inner[j.parent[inner] >= 0]] < inner[j.parent[inner] >= 0])
