"""Topology search host logic (laml_gb300/tree.py, laml_gb300/topology_search.py)
on the CPU: tree operations in treeswift's orders, NNI move listing, the
search loop with a stand-in scorer; the GPU search is in
tests/test_gpu_topology.py."""
import random

import pytest

from laml_gb300 import topology_search as TS
from laml_gb300.tree import find_lcas, read_tree_newick
from oracle import pmm_oracle as O


def test_newick_round_trip_and_preorder():
    nw = "((a:1.0,b:2.0)x:0.5,(c:0.25,(d:1.0,e:3.0):0.125):0.75)r;"
    t = read_tree_newick(nw)
    assert t.newick() == nw
    ours = [v.label for v in t.traverse_preorder()]
    ref = [v.label for v in O.preorder(O.read_newick(nw))]
    assert ours == ref
    post = [v.label for v in t.traverse_postorder()]
    assert post == [v.label for v in O.postorder(O.read_newick(nw))]


def test_resolve_and_suppress():
    t = read_tree_newick("(a,b,c,d,e);")
    t.resolve_polytomies()
    assert all(len(v.children) in (0, 2) for v in t.traverse_preorder())
    assert sorted(v.label for v in t.traverse_leaves()) == list("abcde")
    u = read_tree_newick("(((a:1,b:1):2):3,c:1);")
    u.suppress_unifurcations()
    assert all(len(v.children) != 1 for v in u.traverse_preorder())
    ab = find_lcas(u, [("a", "b")])[0]
    assert ab.edge_length == pytest.approx(5.0)


def test_find_lcas():
    t = read_tree_newick("((a,b)x,((c,d)y,e)z)r;")
    got = [n.label for n in find_lcas(t, [("a", "b"), ("c", "e"), ("a", "d"), ("d", "d"),
                                          ("c", "d")])]
    assert got == ["x", "z", "r", "d", "y"]
    assert find_lcas(t, [("a", "nope")]) == [None]


class _FakeSolver:
    """Scores a tree by how many of a target's clades it has (CPU stand-in
    for the GPU solver; the search logic is what is under test)."""
    target = None

    def __init__(self, treeList, data, prior, params):
        self.trees = list(treeList)
        self.params = dict(params) if params else {'nu': 0.1, 'phi': 0.1}

    @staticmethod
    def clades(nw):
        t = read_tree_newick(nw)
        out = set()
        for v in t.traverse_postorder():
            v.anchors = (frozenset([v.label]) if v.is_leaf()
                         else frozenset().union(*[c.anchors for c in v.children]))
            if not v.is_leaf():
                out.add(v.anchors)
        return out

    def score_tree(self, strategy):
        return float(len(self.clades(self.trees[0]) & self.clades(self.target))), "optimal"

    def get_tree_newick(self):
        return self.trees

    def get_params(self):
        return self.params


def test_nni_moves_listed_and_restored():
    random.seed(4)
    nw = "((((a,b),c),(d,e)),(f,(g,h)));"
    s = TS.Topology_search_batched([nw], _FakeSolver, params={'nu': 0.1, 'phi': 0.1})
    before = s.treeList_obj[0].newick()
    moves = s.list_all_nni(dict(TS.DEFAULT_STRATEGY, local_brlen_opt=False))
    n_internal_nonroot = sum(1 for v in s.treeList_obj[0].traverse_preorder()
                             if not v.is_leaf() and not v.is_root())
    assert len(moves) == 2 * n_internal_nonroot
    # every move undone (children come back appended, as with treeswift)
    assert _FakeSolver.clades(s.treeList_obj[0].newick()) == _FakeSolver.clades(before)
    for topos, _, _ in moves:
        t = read_tree_newick(topos[0])
        assert sorted(v.label for v in t.traverse_leaves()) == list("abcdefgh")
        assert all(len(v.children) in (0, 2) for v in t.traverse_preorder())
        assert _FakeSolver.clades(topos[0]) != _FakeSolver.clades(before)
    assert len({frozenset(_FakeSolver.clades(m[0][0])) for m in moves}) == len(moves)


def test_local_strategy_fixes_all_but_the_move():
    random.seed(1)
    nw = "((((a:1,b:1):1,c:1):1,(d:1,e:1):1):1,(f:1,g:1):1);"
    s = TS.Topology_search([nw], _FakeSolver, params={'nu': 0.2, 'phi': 0.3})
    u = next(v for v in s.treeList_obj[0].traverse_preorder()
             if not v.is_leaf() and not v.is_root() and not v.parent.is_root())
    st = s._local_strategy(u, u.parent, TS.DEFAULT_STRATEGY)
    assert st['fixed_nu'] == 0.2 and st['fixed_phi'] == 0.3
    nfree = len(u.child_nodes()) + len(u.parent.child_nodes()) + 1
    nall = sum(1 for _ in s.treeList_obj[0].traverse_preorder())
    assert len(st['fixed_brlen'][0]) == nall - nfree
    assert all(L == 1.0 for L in st['fixed_brlen'][0].values() if L is not None)


@pytest.mark.parametrize("batched", [False, True])
def test_search_finds_target_with_stand_in_scorer(batched, monkeypatch):
    random.seed(7)
    _FakeSolver.target = "((((a,b),c),d),((e,f),(g,h)));"
    start = "((((a,h),c),g),((e,f),(d,b)));"
    strat = dict(TS.DEFAULT_STRATEGY, local_brlen_opt=False)
    if batched:
        def fake_batch(cands, strats, data, prior, params, group_sites=8, device="cuda"):
            out = []
            for topos in cands:
                sc = _FakeSolver(topos, data, prior, params).score_tree({})[0]
                r = type("R", (), {})()
                r.score, r.newicks, r.params = sc, topos, dict(params)
                out.append(r)
            return out
        import laml_gb300.fastEM_solver as FS
        monkeypatch.setattr(FS, "score_candidate_batch", fake_batch)
        s = TS.Topology_search_batched([start], _FakeSolver, params={'nu': .1, 'phi': .1},
                                       batch_size=7)
    else:
        s = TS.Topology_search([start], _FakeSolver, params={'nu': .1, 'phi': .1})
    trees, score, params = s.search(maxiter=200, nreps=3, strategy=strat)
    assert score == len(_FakeSolver.clades(_FakeSolver.target))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_nni_candidates_equal_encoded_newicks(seed):
    """laml_nni_candidates against the search's own path: swap the Python
    tree, write its newick, encode it.  Every array equal, for every move."""
    import numpy as np
    from laml_gb300 import synth
    from laml_gb300.encoding import encode_newick, nni_candidates
    from laml_gb300.topology_search import Topology_search, encoded_ids
    from laml_gb300.tree import read_tree_newick
    w = synth.pmm_workload(40, 5, 3, 6, 0.5, 0.1, 0.1, seed=seed)
    tree = read_tree_newick(w.newicks[0])
    leaf_index = {c: i for i, c in enumerate(w.leaf_order)}
    ids = encoded_ids(tree, leaf_index)
    et = encode_newick(tree.newick(), w.leaf_order)
    moves, ref = [], []
    for u in tree.traverse_preorder():
        if u.is_leaf() or u.get_parent() is None:
            continue
        v = u.get_parent()
        wn = next(x for x in v.child_nodes() if x is not u)
        for uc in list(u.child_nodes()):
            Topology_search._swap(u, v, uc, wn)
            ref.append(encode_newick(tree.newick(), w.leaf_order))
            Topology_search._unswap(u, v, uc, wn)
            moves.append((ids[id(u)], ids[id(uc)]))
    assert len(moves) == 2 * (et.num_nodes - et.num_leaves - 1)
    cands = nni_candidates(et, moves)
    for c, r in zip(cands, ref):
        for a in ("parent", "child0", "child1", "branch_length", "has_length"):
            np.testing.assert_array_equal(getattr(c, a), getattr(r, a), err_msg=a)


def test_nni_candidates_rejects_bad_moves():
    import numpy as np
    from laml_gb300 import _native as N
    from laml_gb300.encoding import encode_newick, nni_candidates
    et = encode_newick("((a:1,b:1):1,(c:1,d:1):1):0.5;", ["a", "b", "c", "d"])
    root = et.root
    with pytest.raises(N.LamlError):
        nni_candidates(et, [(root, int(et.child0[root]))])   # u may not be the root
    with pytest.raises(N.LamlError):
        nni_candidates(et, [(0, 1)])                          # u must be internal
    u = int(et.child0[root])
    with pytest.raises(N.LamlError):
        nni_candidates(et, [(u, 0 if et.parent[0] != u else 2)])   # not a child of u


@pytest.mark.parametrize("seed", [3, 4])
def test_native_nni_listing_equals_newick_listing(seed):
    """Topology_search_batched.list_all_nni, native (leaf order given) against
    the newick path under the same random seed: the same moves in the same
    order, candidates encoded identically, each candidate's listing-time
    newick rebuilt exactly, and the tree object left with the same child
    orders (the next round's listing reads them)."""
    import copy
    import numpy as np
    from laml_gb300 import synth
    from laml_gb300.encoding import encode_newick_batch
    w = synth.pmm_workload(30, 5, 3, 6, 0.5, 0.1, 0.1, seed=seed)
    strat = dict(TS.DEFAULT_STRATEGY)
    prior = {"Q": w.Q}
    with_order = {"charMtrx": w.rows, "ordered_leaf_labels": [w.leaf_order]}
    without = {"charMtrx": w.rows}
    a = TS.Topology_search_batched([w.newicks[0]], None, data=with_order, prior=prior,
                                   params={"nu": .1, "phi": .2})
    b = TS.Topology_search_batched([w.newicks[0]], None, data=without, prior=prior,
                                   params={"nu": .1, "phi": .2})
    for _ in range(2):   # two rounds: the second starts from the mutated child orders
        random.seed(seed)
        na = a.list_all_nni(strat)
        random.seed(seed)
        nb = b.list_all_nni(strat)
        assert len(na) == len(nb)
        ref = encode_newick_batch([m[0][0] for m in nb], w.leaf_order)
        for k, (x, y) in enumerate(zip(na, nb)):
            assert [n.label for n in x[2]] == [n.label for n in y[2]]
            assert x[1]['fixed_nu'] == y[1]['fixed_nu'] and x[1]['fixed_phi'] == y[1]['fixed_phi']
            assert (x[1]['fixed_brlen'] is None) == (y[1]['fixed_brlen'] is None)
            for f in ("parent", "child0", "child1", "branch_length", "has_length"):
                np.testing.assert_array_equal(getattr(x[3], f), getattr(ref[k], f), err_msg=f)
        for k in (0, len(na) // 2, len(na) - 1):
            assert na[k][4]() == nb[k][0]
        assert a.treeList_obj[0].newick() == b.treeList_obj[0].newick()
