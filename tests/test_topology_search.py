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
