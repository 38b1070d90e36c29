"""Several trees in one EM (EM_solver with a list of trees).

EM_solver (laml_libs/EM_solver.py) keeps one nu and one phi for all of its
trees: the E-step runs on every tree, the M-step takes phi from the leaves of
all trees (307-326), solves every branch length and one nu over the branches
of all trees (327-407), and the EM stops on the summed log-likelihood
(461-512).  With ultra_constr the equalities of each tree are joined by
equalities that give every tree's root (its own branch included) the same
height (ultrametric_constr, 53-89: rows trees[0].root - tree.root).

Here the trees are joined into one binary tree for the device: a caterpillar
of k - 1 joining nodes above the k roots, each joining node's own branch
fixed at length 0.  In the exact (EM_solver) model a branch of length 0 is
transparent -- P(0 -> 0) = 1 and every other transition from state 0 is 0 --
so the progenitor's state 0 reaches every original root unchanged:

* the joined site likelihood is the product of the trees' site likelihoods,
  and every original node's posterior and expected counts are its own
  tree's;
* the joined tree's M-step (fixed branches excluded from the nu sums, phi
  over all leaves) is EM_solver's joint M-step;
* under the ultrametric M-step the joining nodes' equalities (two children
  at one height, fixed zero branches tying heights together) are exactly
  the reference's root rows: root height + root branch equal for all trees.

Leaves of tree t keep their own rows in a dataset of the trees' rows
concatenated, so the counts of '?' entries sum over the trees as the
reference's phi does.  The fastEM model floors 1 - e^{-d} at EPS and is not
transparent at d = 0: joining is for the exact model only.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np

from .encoding import EncodedTree


def join_forest(trees: Sequence[EncodedTree]) -> Tuple[EncodedTree, List[np.ndarray], np.ndarray]:
    """The joined tree, the joined id of every node of each tree, and the
    joined ids of the joining nodes (fixed at length 0).  Leaves come first
    (tree 0's, tree 1's, ...), then the joining nodes top-down, then each
    tree's internal nodes in their own order, so parents precede children."""
    k = len(trees)
    if k == 1:
        t = trees[0]
        return t, [np.arange(t.num_nodes)], np.zeros(0, np.int64)
    n_tot = sum(t.num_leaves for t in trees)
    V = k - 1
    n_int = sum(t.num_nodes - t.num_leaves for t in trees)
    N = n_tot + V + n_int
    maps = []
    lo, io = 0, n_tot + V
    for t in trees:
        m = np.empty(t.num_nodes, np.int64)
        m[:t.num_leaves] = lo + np.arange(t.num_leaves)
        m[t.num_leaves:] = io + np.arange(t.num_nodes - t.num_leaves)
        lo += t.num_leaves
        io += t.num_nodes - t.num_leaves
        maps.append(m)
    parent = np.full(N, -1, np.int32)
    c0 = np.full(N, -1, np.int32)
    c1 = np.full(N, -1, np.int32)
    bl = np.zeros(N, np.float64)
    has = np.ones(N, bool)
    labels = [""] * N
    for t, m in zip(trees, maps):
        par = np.asarray(t.parent)
        nz = par >= 0
        parent[m[nz]] = m[par[nz]]
        inner = np.asarray(t.child0) >= 0
        c0[m[inner]] = m[np.asarray(t.child0)[inner]]
        c1[m[inner]] = m[np.asarray(t.child1)[inner]]
        bl[m] = t.branch_length
        has[m] = t.has_length
        if t.labels is not None:
            for u in range(t.num_nodes):
                labels[m[u]] = t.labels[u]
    joins = n_tot + np.arange(V)
    roots = [int(m[t.root]) for t, m in zip(trees, maps)]
    for j in range(V):
        v = int(joins[j])
        a = roots[j]
        b = int(joins[j + 1]) if j + 1 < V else roots[j + 1]
        c0[v], c1[v] = b, a   # child1: the first in newick order
        parent[a] = v
        parent[b] = v
        bl[v] = 0.0
        labels[v] = f"join_{j}"
    joined = EncodedTree(N, n_tot, parent, c0, c1, bl, has, labels)
    return joined, maps, joins
