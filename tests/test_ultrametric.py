"""Ultrametric-constrained M-step (EM_solver.Mstep with ultra_constr_cache,
laml_libs/EM_solver.py:53-89, 349-366), CPU side.

* the oracle's constraint rows restate EM_solver.ultrametric_constr;
* the oracle's ultrametric EM, brute-forced over the 15 rooted topologies of
  the four-leaf case of unit_tests_TopoSearch.py test_10, reaches that test's
  pre-computed optimum (nllh_bf = 7.0063474330891236) to the test's own
  places=4;
* laml_ultra_order (the device solve's depth schedule) on the host.
"""
import ctypes as C

import numpy as np
import pytest

from laml_gb300 import _native as N
from laml_gb300.encoding import encode_newick
from oracle import pmm_oracle as O
from tests.helpers import rooted_topologies, ultrametric_cases


def _path_lengths(tree, d):
    """Root-to-leaf path lengths below the root (the root's branch excluded)."""
    out = []
    for leaf in range(tree.num_leaves):
        s, x = 0.0, leaf
        while tree.parent[x] >= 0:
            s += d[x]
            x = tree.parent[x]
        out.append(s)
    return np.array(out)


def test_constraint_rows_restate_ultrametric_constr():
    tr = O.parse_tree("((a:1,b:1):1,(c:1,d:1):1):0.5;", ["a", "b", "c", "d"])
    d = tr.branch_lengths.copy()
    M, b, free = O.ultrametric_constraints(tr, np.ones(7, bool), d)
    # one row per internal node: (a, b), (c, d), and the root's two paths
    assert M.shape == (3, 7) and np.all(b == 0)
    # every solution of M x = 0 gives equal root-to-leaf paths
    rng = np.random.default_rng(1)
    from scipy.linalg import null_space
    Z = null_space(M)
    for _ in range(5):
        x = Z @ rng.normal(size=Z.shape[1])
        dd = np.zeros(7)
        dd[free] = x
        p = _path_lengths(tr, dd)
        assert np.ptp(p) < 1e-12


def test_constraint_rows_with_fixed_branches():
    # leaf a's branch fixed at 0.7: the cherry (a, b) forces d_b = 0.7
    tr = O.parse_tree("((a:0.7,b:1):1,(c:1,d:1):1):0.5;", ["a", "b", "c", "d"])
    mask = np.ones(7, bool)
    mask[0] = False
    M, b, free = O.ultrametric_constraints(tr, mask, tr.branch_lengths)
    assert 0 not in free
    x = np.full(len(free), 0.3)
    col = {v: i for i, v in enumerate(free)}
    x[col[1]] = 0.7
    x[col[2]] = x[col[3]] = 0.3
    # (a, b) at height 0.7, (c, d) at 0.3: parents' branches 0.3 and 0.7
    ab = tr.parent[0]
    cd = tr.parent[2]
    x[col[ab]] = 0.3
    x[col[cd]] = 0.7
    assert np.allclose(M @ x, b)


@pytest.mark.slow
def test_oracle_ultrametric_bruteforce_reaches_reference_optimum():
    (case,) = ultrametric_cases()
    leaves = case["leaves"]
    best = np.inf
    for top in rooted_topologies(leaves):
        tr = O.parse_tree(top + ";", leaves)
        enc = O.recode([case["msa"][c] for c in leaves], case["Q"], compat=False)
        prob = O.Problem(tr, enc, False)
        post = O.treeswift_postorder_ids(tr)
        x, nu, phi = O.exact_initials(tr, [None] * len(post), 1)
        d = np.empty(len(tr.parent))
        for i, u in enumerate(post):
            d[u] = x[i]
        r = O.em_exact(prob, d, nu, phi, ultra=True)
        assert r.status == "optimal"
        assert np.ptp(_path_lengths(tr, r.d)) < 1e-9
        assert np.all(r.d >= O.DMIN - 1e-12) and np.all(r.d <= O.DMAX + 1e-12)
        best = min(best, -r.llh)
    # unit_tests_TopoSearch.py test_9/test_10 compare with places=4
    assert round(best - case["nllh_bf"], 4) == 0


def test_oracle_ultrametric_infeasible_and_dropped_rows():
    S = np.ones((5, 6))
    # a fixed at 20: its sibling b would need d_b = 20 > dmax -> infeasible
    tr = O.parse_tree("((a:20,b:2):1,c:1):0.5;", ["a", "b", "c"])
    mask = np.ones(5, bool)
    mask[0] = False
    d, ok = O.ultrametric_d(S, 0.1, tr.branch_lengths, mask, tr)
    assert not ok
    # a at 1 and b at 2, both fixed: the row between two constants is
    # dropped (EM_solver.py:70-72), so the problem is feasible
    tr = O.parse_tree("((a:1,b:2):1,c:1):0.5;", ["a", "b", "c"])
    mask = np.ones(5, bool)
    mask[0] = mask[1] = False
    M, b, free = O.ultrametric_constraints(tr, mask, tr.branch_lengths)
    assert M.shape[0] == 1
    d, ok = O.ultrametric_d(S, 0.1, tr.branch_lengths, mask, tr)
    assert ok


def _order(newick):
    t = encode_newick(newick)
    out = np.zeros(2 * t.num_nodes + 2, np.int32)
    w = N.i64()
    rc = N.lib().laml_ultra_order(np.ascontiguousarray(t.parent, np.int32).ctypes.data,
                                  t.num_nodes, out.ctypes.data, out.size, C.byref(w))
    return t, rc, out, w.value


@pytest.mark.parametrize("nw", ["((a,b),(c,d));", "(((a,b),c),d);", "((a,(b,(c,(d,e)))),f);",
                                "(a,b);"])
def test_ultra_order_groups_nodes_by_depth(nw):
    t, rc, out, written = _order(nw)
    assert rc == 0
    L = out[0]
    off = out[1:L + 2]
    ids = out[L + 2:L + 2 + t.num_nodes]
    assert written == t.num_nodes + L + 2
    assert off[0] == 0 and off[-1] == t.num_nodes
    assert sorted(ids.tolist()) == list(range(t.num_nodes))
    depth = np.zeros(t.num_nodes, int)
    for l in range(L):
        for x in ids[off[l]:off[l + 1]]:
            depth[x] = l
    assert ids[0] == t.root and off[1] == 1
    for x in range(t.num_nodes):
        if t.parent[x] >= 0:
            assert depth[x] == depth[t.parent[x]] + 1


def test_ultra_order_errors():
    out = np.zeros(16, np.int32)
    w = N.i64()
    lib = N.lib()
    two_roots = np.array([-1, -1, 0], np.int32)
    assert lib.laml_ultra_order(two_roots.ctypes.data, 3, out.ctypes.data, 16, C.byref(w)) == -1
    three_kids = np.array([-1, 0, 0, 0], np.int32)
    assert lib.laml_ultra_order(three_kids.ctypes.data, 4, out.ctypes.data, 16, C.byref(w)) == -6
    one_kid = np.array([-1, 0], np.int32)
    assert lib.laml_ultra_order(one_kid.ctypes.data, 2, out.ctypes.data, 16, C.byref(w)) == -6
    short = np.array([-1, 0, 0], np.int32)
    assert lib.laml_ultra_order(short.ctypes.data, 3, out.ctypes.data, 7, C.byref(w)) == -1
