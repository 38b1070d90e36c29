"""Seeded synthetic PMM workloads (the reference ships no generator of its own).

* Yule trees: successive uniform leaf splits; branch lengths ~ Exp(mean) with
  a floor (0.006 = dmin + 0.001 of laml_libs/core_constants.py:7).
* Characters simulated down the tree as laml_libs/sim_lib.py:64-105
  (simulate_seqs): mutation rate 1, from state 0 the child is 0 w.p.
  e^{-d(1+nu)}, state a w.p. q_a e^{-nu d}(1-e^{-d}), silenced w.p.
  1-e^{-nu d}; a mutated state persists w.p. e^{-nu d}; silencing absorbs;
  leaves drop out w.p. phi unless silenced; silenced and dropped -> '?'.
* Priors: per site M_k ~ U{lo..hi} states with q ~ Dirichlet(alpha).
* NNI neighbours: swap a child of an internal non-root node with its sibling.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Optional, Tuple

import numpy as np


@dataclass
class SimTree:
    parent: np.ndarray      # int64[N], -1 root
    children: List[List[int]]
    length: np.ndarray      # float64[N] (root edge included)
    labels: List[str]       # leaf names ('' for internal)
    root: int

    def newick(self) -> str:
        out = []
        st = [(self.root, 0)]
        while st:
            u, k = st.pop()
            ch = self.children[u]
            if not ch:
                out.append(f"{self.labels[u]}:{float(self.length[u])!r}")
                continue
            if k == 0:
                out.append("(")
            if k < len(ch):
                if k > 0:
                    out.append(",")
                st.append((u, k + 1))
                st.append((ch[k], 0))
            else:
                out.append(f"):{float(self.length[u])!r}")
        return "".join(out) + ";"

    def leaves(self) -> List[int]:
        return [u for u in range(len(self.parent)) if not self.children[u]]


def yule_tree(n_leaves: int, rng: np.random.Generator, mean_length: float = 0.1,
              floor: float = 0.006) -> SimTree:
    parent = [-1, 0, 0]
    children = [[1, 2], [], []]
    leaves = [1, 2]
    while len(leaves) < n_leaves:
        k = int(rng.integers(len(leaves)))
        u = leaves[k]
        a, b = len(parent), len(parent) + 1
        parent += [u, u]
        children += [[], []]
        children[u] = [a, b]
        leaves[k] = a
        leaves.append(b)
    N = len(parent)
    length = np.maximum(rng.exponential(mean_length, size=N), floor)
    labels = [""] * N
    for i, u in enumerate(sorted(leaves)):
        labels[u] = f"c{i}"
    return SimTree(np.asarray(parent), children, length, labels, 0)


def dirichlet_priors(n_sites: int, m_lo: int, m_hi: int, alpha: float,
                     rng: np.random.Generator) -> List[dict]:
    Q = []
    for _ in range(n_sites):
        m = int(rng.integers(m_lo, m_hi + 1))
        q = rng.dirichlet(np.full(m, alpha))
        q = np.maximum(q, 1e-12)
        q = q / q.sum()
        Q.append({j + 1: float(q[j]) for j in range(m)})
    return Q


def simulate(tree: SimTree, Q: List[dict], nu: float, phi: float, rng: np.random.Generator,
             mu: float = 1.0):
    """Leaf character rows (dict label -> list of int | '?')."""
    K = len(Q)
    states = [np.asarray(list(q.keys())) for q in Q]
    cum = [np.cumsum(np.asarray(list(q.values()))) for q in Q]
    SIL = -1
    seq = {}
    st = [tree.root]
    order = []
    while st:
        u = st.pop()
        order.append(u)
        st.extend(tree.children[u])
    z = np.zeros(K, np.int64)
    for u in order:
        d = tree.length[u] * mu
        p = math.exp(-d)
        pnu = p ** nu
        par = seq[tree.parent[u]] if tree.parent[u] >= 0 else z
        r = rng.random(K)
        child = par.copy()
        # from state 0: 0 | mutated | silenced
        p00 = p ** (nu + 1)
        pm = pnu * (1 - p)
        zero = par == 0
        to_mut = zero & (r >= p00) & (r < p00 + pm)
        to_sil0 = zero & (r >= p00 + pm)
        for c in np.flatnonzero(to_mut):
            x = (r[c] - p00) / pm
            j = int(np.searchsorted(cum[c], x * cum[c][-1], side="right"))
            child[c] = states[c][min(j, len(states[c]) - 1)]
        child[to_sil0] = SIL
        mut = par > 0
        child[mut & (r >= pnu)] = SIL
        seq[u] = child
    rows = {}
    for u in tree.leaves():
        s = seq[u]
        drop = rng.random(K) < phi
        rows[tree.labels[u]] = ["?" if (s[c] == SIL or drop[c]) else int(s[c]) for c in range(K)]
    return rows


def nni_neighbour(tree: SimTree, rng: np.random.Generator) -> SimTree:
    """A random nearest-neighbour interchange: for an internal non-root node v
    with sibling w, swap one child of v with w (lengths travel with their
    subtrees)."""
    N = len(tree.parent)
    cand = [v for v in range(N) if tree.children[v] and tree.parent[v] >= 0]
    v = cand[int(rng.integers(len(cand)))]
    u = int(tree.parent[v])
    w = [c for c in tree.children[u] if c != v][0]
    k = int(rng.integers(2))
    x = tree.children[v][k]
    children = [list(c) for c in tree.children]
    parent = tree.parent.copy()
    children[v][k] = w
    children[u][children[u].index(w)] = x
    parent[w] = v
    parent[x] = u
    return SimTree(parent, children, tree.length.copy(), tree.labels, tree.root)


@dataclass
class Workload:
    newicks: List[str]
    rows: dict
    Q: List[dict]
    leaf_order: List[str]
    nu: float
    phi: float


def pmm_workload(n_leaves: int, n_sites: int, m_lo: int, m_hi: int, alpha: float, nu: float,
                 phi: float, seed: int, n_trees: int = 1, nni: bool = False) -> Workload:
    """One Yule tree (+ n_trees-1 NNI neighbours when ``nni``) and a character
    matrix simulated on the first tree."""
    rng = np.random.default_rng(seed)
    t = yule_tree(n_leaves, rng)
    Q = dirichlet_priors(n_sites, m_lo, m_hi, alpha, rng)
    rows = simulate(t, Q, nu, phi, rng)
    trees = [t]
    if nni:
        trees += [nni_neighbour(t, rng) for _ in range(n_trees - 1)]
    else:
        trees += [yule_tree(n_leaves, rng) for _ in range(n_trees - 1)]
    leaf_order = [t.labels[u] for u in sorted(t.leaves())]
    return Workload([x.newick() for x in trees], rows, Q, leaf_order, nu, phi)


def workload_config(name: str, seed: int = 0) -> Workload:
    """The workloads used by the benchmark and the parity tests."""
    if name == "fixed250":      # 250 leaves x 30 sites, M~U{5..30}, Dir(0.5)
        return pmm_workload(250, 30, 5, 30, 0.5, 0.1, 0.15, seed)
    if name == "nni512":        # 512 NNI neighbours of a 1000-leaf tree, 40 sites
        return pmm_workload(1000, 40, 5, 50, 0.5, 0.1, 0.15, seed, n_trees=512, nni=True)
    if name == "grad4096":
        return pmm_workload(4096, 100, 10, 100, 0.3, 0.05, 0.1, seed)
    if name == "large50k":
        return pmm_workload(50000, 300, 20, 100, 0.2, 0.1, 0.2, seed)
    raise KeyError(name)
