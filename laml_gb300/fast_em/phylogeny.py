"""Mirror of fast_em/phylogeny.py: the Phylogeny dataclass, build_phylogeny
(fast_em/phylogeny.py:48-114) and parse_newick (116-161).

pandas and treeswift are not needed: the character matrix may be given as
``(row_labels, int matrix)`` or as ``{label: [int | '?', ...]}`` and the
priors as ``{(site, state): prob}`` or a list of per-site dicts.  The newick
parser is the engine's C++ encoder (treeswift preorder numbering).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import networkx as nx
import numpy as np

from ..encoding import char_matrix, encode_newick


@dataclass
class Phylogeny:
    num_leaves: int
    num_characters: int
    max_alphabet_size: int
    root: int
    tree: Any                      # networkx.DiGraph
    character_matrix: np.ndarray   # int32 (num_leaves, num_characters)
    mutation_priors: np.ndarray    # float32 (num_characters, max_alphabet_size)


@dataclass
class PhylogenyOptimization:
    phylogeny: Phylogeny
    branch_lengths: np.ndarray
    model_parameters: np.ndarray
    inside_log_likelihoods: Any = None


def _matrix(character_matrix):
    if isinstance(character_matrix, dict):
        labels = list(character_matrix)
        return labels, char_matrix([character_matrix[x] for x in labels])
    labels, mat = character_matrix
    return list(labels), np.asarray(mat, np.int64)


def _prior_lookup(mutation_priors):
    if isinstance(mutation_priors, dict):
        return lambda c, s: mutation_priors[(c, s)]
    return lambda c, s: mutation_priors[c][s]


def build_phylogeny(tree: nx.DiGraph, num_leaves: int, character_matrix, mutation_priors) -> Phylogeny:
    """fast_em/phylogeny.py:48-114: recode each column's observed non-zero
    states to 1..k in sorted order, build the dense float32 prior table of the
    observed states (no renormalisation), and order the rows by leaf index
    (``tree.nodes[leaf]['label']`` names the row).  A missing prior raises
    KeyError (the reference logs and exits, phylogeny.py:91-93)."""
    roots = [v for v in tree.nodes() if tree.in_degree(v) == 0]
    if len(roots) != 1:
        raise ValueError("The tree has more than one root.")
    labels, mat = _matrix(character_matrix)
    mat = np.where(mat < 0, -1, mat)
    n_rows, K = mat.shape
    rec = mat.copy()
    maps = []
    kmax = 0
    for c in range(K):
        valid = sorted(set(int(x) for x in mat[:, c]) - {-1, 0})
        kmax = max(kmax, len(valid))
        m = {o: i + 1 for i, o in enumerate(valid)}
        maps.append(valid)
        for i in range(n_rows):
            if mat[i, c] > 0:
                rec[i, c] = m[int(mat[i, c])]
    look = _prior_lookup(mutation_priors)
    pri = np.zeros((K, kmax), np.float32)
    for c in range(K):
        for j, o in enumerate(maps[c]):
            try:
                pri[c, j] = look(c, o)
            except KeyError:
                raise KeyError(f"Missing mutation prior for character {c}, state {o}")
    row_of = {x: i for i, x in enumerate(labels)}
    order = np.zeros(num_leaves, np.int64)
    for v in tree.nodes():
        if tree.out_degree(v) == 0:
            order[v] = row_of[tree.nodes[v]["label"]]
    return Phylogeny(num_leaves, K, kmax, roots[0], tree, rec[order].astype(np.int32), pri)


def tree_to_networkx(et) -> nx.DiGraph:
    """An EncodedTree as the networkx DiGraph of parse_tree / parse_newick:
    nodes 0..N-1 with 'label' and 'branch_length', edges in successor order."""
    g = nx.DiGraph()
    for i in range(et.num_nodes):
        g.add_node(i, label=et.labels[i],
                   branch_length=float(et.branch_length[i]) if et.has_length[i] else None)
    for i in range(et.num_nodes):
        if et.child0[i] >= 0:
            g.add_edge(i, int(et.child0[i]))
            g.add_edge(i, int(et.child1[i]))
    return g


def parse_newick(newick: str):
    """fast_em/phylogeny.py:116-161: (DiGraph with leaves 0..n-1, n)."""
    if "(" not in newick and not newick.strip().endswith(";"):
        with open(newick) as f:
            newick = f.read()
    et = encode_newick(newick)
    return tree_to_networkx(et), et.num_leaves
