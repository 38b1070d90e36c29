"""Adapters from the reference's dense fast_em arrays to engine encodings."""
from __future__ import annotations

import numpy as np

from ..encoding import EncodedTree, encode_dataset


def as_numpy(x, dtype=None):
    if hasattr(x, "detach"):
        x = x.detach().cpu().numpy()
    a = np.asarray(x)
    return a.astype(dtype) if dtype is not None else a


def tree_from_networkx(g) -> EncodedTree:
    """nx.DiGraph with nodes 0..N-1 (leaves 0..n-1, EMOptimizer's
    convention, fast_em/laml.py:207-251) -> EncodedTree (children in
    successor order)."""
    N = g.number_of_nodes()
    par = np.full(N, -1, np.int32)
    c0 = np.full(N, -1, np.int32)
    c1 = np.full(N, -1, np.int32)
    n = 0
    for u in range(N):
        ch = list(g.successors(u))
        if not ch:
            n += 1
            continue
        if len(ch) != 2:
            raise ValueError("the PMM engine needs a binary tree (node %d has %d children)"
                             % (u, len(ch)))
        c0[u], c1[u] = ch
        par[ch[0]] = u
        par[ch[1]] = u
    labels, bl, has = [], np.zeros(N), np.zeros(N, bool)
    for u in range(N):
        a = g.nodes[u] if u in g.nodes else {}
        labels.append(str(a.get("label", u)))
        if a.get("branch_length") is not None:
            bl[u] = float(a["branch_length"])
            has[u] = True
    if np.any(c0[:n] >= 0) or np.any(c0[n:] < 0):
        raise ValueError("leaves must be numbered 0..n-1")
    return EncodedTree(N, n, par, c0, c1, bl, has, labels)


def tree_from_arrays(num_nodes, leaves, internal_postorder, internal_postorder_children):
    """The topology arrays of calc.compute_E_step (calculations.py:507-520)."""
    N = int(num_nodes)
    leaves = as_numpy(leaves).astype(np.int64)
    ip = as_numpy(internal_postorder).astype(np.int64)
    ipc = as_numpy(internal_postorder_children).astype(np.int64)
    par = np.full(N, -1, np.int32)
    c0 = np.full(N, -1, np.int32)
    c1 = np.full(N, -1, np.int32)
    for (u, _), (v, w) in zip(ip, ipc):
        c0[u], c1[u] = v, w
        par[v] = u
        par[w] = u
    n = len(leaves)
    return EncodedTree(N, n, par, c0, c1, np.zeros(N), np.zeros(N, bool),
                       [str(i) for i in range(N)])


def dataset_from_dense(mutation_priors, character_matrix, group_sites=8):
    """Recoded (n, K) int matrix + dense (K, M) priors of build_phylogeny ->
    the engine layout.  Column c's states are 1..k_c with priors
    mutation_priors[c, :k_c]; padded columns are inert and dropped."""
    mp = as_numpy(mutation_priors, np.float64)
    cm = as_numpy(character_matrix).astype(np.int64)
    cm = np.where(cm < 0, -1, cm).astype(np.int32)
    K = cm.shape[1]
    Q = []
    for c in range(K):
        st = sorted(set(int(x) for x in cm[:, c]) - {-1, 0})
        Q.append({s: float(np.float32(mp[c, s - 1])) for s in st})
    return encode_dataset(cm, Q, compat=True, group_sites=group_sites)
