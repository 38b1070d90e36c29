"""Input formats feeding the encoder: the reference's character-matrix and
prior readers (laml_libs/sequence_lib.py:100-363) and writer (78-92), and
the collapsing of identical sequences before a run with their return as
polytomies after it (dedup / add_dup, sequence_lib.py:10-76).

``read_sequences`` returns (charMtrx, site_names) with charMtrx =
{cell: [int | '?']}; ``read_priors`` returns Q = [{state: prob}] per site
(CSV ``site,state,prob`` with an optional header and optional 'r'-prefixed
site names, or a pickled {site: {state: prob}} dict where state 0 gets prior
0).  These feed ``problem.dataset_from_rows`` / ``fastEM_solver``.
"""
from __future__ import annotations

import pickle
from collections import defaultdict
from typing import Dict, List, Optional, Sequence, Tuple

from .tree import Node, Tree, read_tree_newick

RECOGNIZED_MISSING = {"-", "?", "-1"}   # sequence_lib.py:8
DMIN = 0.005   # laml_libs/core_constants.py: dmin


def _is_missing(seen, x):
    if x in seen or x in RECOGNIZED_MISSING or x.isalpha():
        return True
    try:
        return int(x) < 0
    except ValueError:
        return False


def read_char_matrix(path: str, delimiter: str = ",", masked_symbol: Optional[str] = None,
                     replace_mchar: str = "?") -> Tuple[Dict[str, list], List[str]]:
    """sequence_lib.read_charMtrx (sequence_lib.py:139-175)."""
    seen = {masked_symbol} if masked_symbol is not None else set()
    D = {}
    with open(path) as f:
        site_names = f.readline().strip().split(delimiter)
        if site_names[0] == "cell_name" or "cell" in site_names[0]:
            site_names = site_names[1:]
        for line in f:
            parts = line.strip().split(delimiter)
            if len(parts) < 2:
                continue
            seq = []
            for x in parts[1:]:
                if _is_missing(seen, x):
                    seen.add(x)
                    seq.append(replace_mchar if replace_mchar is not None else x)
                else:
                    seq.append(int(x))
            D[parts[0]] = seq
    return D, site_names


def read_sequences(path: str, filetype: str = "charMtrx", delimiter: str = ",",
                   masked_symbol: Optional[str] = None, suppress_warnings: bool = False,
                   replace_mchar: str = "?"):
    if filetype != "charMtrx":
        raise ValueError("only the charMtrx format is supported")
    return read_char_matrix(path, delimiter, masked_symbol, replace_mchar)


def read_priors(path: str, msa: Optional[dict] = None,
                site_names: Optional[Sequence[str]] = None) -> List[Dict[int, float]]:
    """sequence_lib.read_priors: CSV (324-355) or pickle (261-322, the
    site-name matching branch excepted: keys are taken in sorted order)."""
    ext = path.strip().split(".")[-1]
    if ext in ("pkl", "pickle"):
        with open(path, "rb") as f:
            priors = pickle.load(f)
        Q = []
        for i in sorted(priors.keys()):
            q = {int(x): priors[i][x] for x in priors[i]}
            q[0] = 0
            Q.append(q)
        return Q
    Q, Qi, seen = [], {}, set()
    with open(path) as f:
        lines = f.readlines()
    tokens = lines[0].split(",")
    if not tokens[1].isnumeric() and not tokens[2].isnumeric():
        lines = lines[1:]
    charname_is_str = not lines[0].split(",")[0].isnumeric()
    for line in lines:
        site, state, prob = line.strip().split(",")
        site = int(site[1:]) if charname_is_str else int(site)
        if site not in seen:
            if seen:
                Q.append(Qi)
                Qi = {}
            seen.add(site)
        Qi[int(state)] = float(prob)
    Q.append(Qi)
    return Q


def write_sequences(char_mtrx: dict, nsites: int, path: str, delimiter: str = ","):
    """sequence_lib.write_sequences (sequence_lib.py:78-92)."""
    with open(path, "w") as f:
        f.write("cell" + "".join(delimiter + "r" + str(i) for i in range(nsites)) + "\n")
        for cell, seq in char_mtrx.items():
            f.write(cell + "".join(delimiter + str(x) for x in seq) + "\n")


def _without_leaves(tree: Tree, labels) -> Tree:
    """A copy of ``tree`` without the leaves named in ``labels``: internal
    nodes left without children go too, and nodes left with one child are
    suppressed (their edge length added to the child's), as treeswift's
    extract_tree_without(labels, suppress_unifurcations=True) leaves it."""
    drop = set(labels)
    new = {}
    for v in tree.traverse_postorder():   # children before parents
        if v.is_leaf():
            if v.label in drop:
                continue
        else:
            kids = [new[c] for c in v.children if c in new]
            if not kids:
                continue
        c = Node(v.label, v.edge_length)
        if not v.is_leaf():
            for k in (new[x] for x in v.children if x in new):
                c.add_child(k)
        new[v] = c
    if tree.root not in new:
        return Tree(Node())
    out = Tree(new[tree.root])
    out.suppress_unifurcations()
    return out


def dedup(char_mtrx: Dict[str, list], input_tree_strings: Sequence[str]):
    """sequence_lib.dedup (sequence_lib.py:10-53): cells with identical
    sequences are grouped (first-seen order); the first cell of each group
    represents it and the others are pruned from every tree.  Returns
    (has_dup, dup_map {representative: [others]}, char_mtrx -- returned
    whole, as the reference does -- and the pruned newick strings)."""
    seq_to_taxa = defaultdict(list)
    for taxon, seq in char_mtrx.items():
        seq_to_taxa[tuple(seq)].append(taxon)
    if len(seq_to_taxa) == len(char_mtrx):
        return False, {}, char_mtrx, list(input_tree_strings)
    dup_map = {g[0]: g[1:] for g in seq_to_taxa.values() if len(g) > 1}
    out = []
    for s in input_tree_strings:
        t = read_tree_newick(s)
        for rep in dup_map:
            t = _without_leaves(t, dup_map[rep])
        out.append(t.newick())
    return True, dup_map, char_mtrx, out


def add_dup(input_tree_strings: Sequence[str], dup_map: Dict[str, List[str]]) -> List[str]:
    """sequence_lib.add_dup (sequence_lib.py:55-76): each representative
    leaf is replaced by a node "node_dummy_<rep>" carrying the leaf's edge
    length (appended as its parent's last child), under which the leaf and
    its duplicates hang with length dmin."""
    out = []
    for s in input_tree_strings:
        t = read_tree_newick(s)
        leaves = {v.label: v for v in t.traverse_leaves()}
        for rep, dups in dup_map.items():
            node = leaves.get(rep)
            if node is None:
                continue
            p = node.get_parent()
            dummy = Node(None, node.edge_length)
            p.remove_child(node)
            p.add_child(dummy)
            node.edge_length = DMIN
            dummy.add_child(node)
            dummy.label = f"node_dummy_{rep}"
            for taxon in dups:
                dummy.add_child(Node(taxon, DMIN))
        out.append(t.newick())
    return out
