"""Posterior annotations (laml_libs/runner.py:367-435) from the GPU E-step.

For each node and site, P(v = 0 | D) and P(v = silenced | D) come from the
exact-model (EM_solver) outside pass on the GPU (laml_outside with
LAML_OUT_POSTERIORS); the per-branch expected mutation counts S1 + S2 + S4
(C0a + C0s + Cas summed over sites) become the branch lengths of the
annotated tree.  The alpha-clade labels (ML_solver.az_partition,
ML_solver.py:125-154) and the string format (runner.format_posterior) are
host-side integer work.

The posteriors are FP32: a probability within ~1e-6 of a rounding boundary
of the 2-decimal output can round the other way than the FP64 reference.
"""
from __future__ import annotations

import math
from typing import Dict, List, Sequence

import numpy as np

from .encoding import char_matrix, encode_dataset, encode_newick
from .engine import DeviceBatch


def format_posterior(p0, p_minus_1, p_alpha, alpha, q):
    """runner.format_posterior (runner.py:368-389)."""
    if p0 == 1:
        return "0"
    elif p_minus_1 == 1:
        return "-1"
    elif p_alpha == 1:
        return alpha
    out = ""
    if p0 > 0:
        out += "0:" + str(p0)
    if p_minus_1 > 0:
        if out != "":
            out += "/"
        out += "-1:" + str(p_minus_1)
    if p_alpha > 0:
        if out != "":
            out += "/"
        if alpha == "?":
            out += "/".join([str(y) + ":" + str(round(p_alpha * q[y], 3)) for y in q
                             if round(p_alpha * q[y], 3) > 0])
        else:
            out += alpha + ":" + str(p_alpha)
    return out


def az_labels(et, rows: Sequence[Sequence]):
    """ML_solver.az_partition: per (node, site) 'z', '?' or the observed
    state (original coding) of the node's alpha-clade."""
    N, n = et.num_nodes, et.num_leaves
    K = len(rows[0])
    lab = [[None] * K for _ in range(N)]
    order = []
    st = [et.root]
    while st:   # treeswift's preorder: the last child in newick order (child0) first
        u = st.pop()
        order.append(u)
        if et.child0[u] >= 0:
            st.append(int(et.child1[u]))
            st.append(int(et.child0[u]))
    for u in reversed(order):
        if u < n:
            for c in range(K):
                x = rows[u][c]
                lab[u][c] = "z" if x == 0 else ("?" if (x == "?" or (isinstance(x, int) and x < 0))
                                                else x)
        else:
            a, b = lab[int(et.child0[u])], lab[int(et.child1[u])]
            for c in range(K):
                S = {a[c], b[c]}
                R = S - {"z", "?"}
                lab[u][c] = "z" if ("z" in S or len(R) > 1) else (next(iter(R)) if R else "?")
    return lab, order


def annotation_lines(et, rows: Sequence[Sequence], Q: List[dict], p0, p1, mut):
    """The runner's annotation output (runner.py:391-430) from per-node
    posteriors: ``p0`` = P(v = 0 | D), ``p1`` = P(v = silenced | D) as [N, K]
    probabilities (original site order), ``mut`` = the expected mutations on
    each node's branch (S1 + S2 + S4 summed over sites).  Returns (annotated
    newick, [(label, posterior string)]) in the runner's order: a new root
    'I0' above the tree (runner.py:396-405), unlabelled or repeated labels
    replaced by I<k> in preorder, branch lengths = round(mut, 3)."""
    lab, order = az_labels(et, rows)
    K = len(rows[0])
    names = {}
    seen = set()
    idx = 1
    for u in order:
        nm = et.labels[u]
        if nm.startswith("node_") or nm in seen:
            nm = "I" + str(idx)
            idx += 1
        seen.add(nm)
        names[u] = nm
    mut = np.round(np.asarray(mut, np.float64), 3)
    parent = {int(et.child0[u]): u for u in order if et.child0[u] >= 0}
    parent.update({int(et.child1[u]): u for u in order if et.child0[u] >= 0})
    # alpha of '?' nodes inherits the parent's when the parent is not 'z'
    for u in order:
        if u in parent:
            pu = parent[u]
            for c in range(K):
                if lab[u][c] == "?" and lab[pu][c] != "z":
                    lab[u][c] = lab[pu][c]

    def length(x):   # the tree writer prints an integral length without ".0"
        x = float(x)
        return str(int(x)) if x.is_integer() else str(x)

    out = []   # newick, children in newick order (child1, then child0); no recursion
    st = [(et.root, 0)]
    while st:
        u, k = st.pop()
        if et.child0[u] >= 0 and k < 2:
            out.append("(" if k == 0 else ",")
            st.append((u, k + 1))
            st.append((int(et.child1[u] if k == 0 else et.child0[u]), 0))
            continue
        if et.child0[u] >= 0:
            out.append(")")
        out.append(f"{names[u]}:{length(mut[u])}")
    tree_line = "(" + "".join(out) + ")I0;"
    lines = [("I0", ",".join(["0"] * K))]
    for u in order:
        parts = []
        for c in range(K):
            a0 = round(float(p0[u, c]), 2)
            a1 = round(float(p1[u, c]), 2)
            aa = round(1 - a0 - a1, 2)
            parts.append(format_posterior(a0, a1, aa, str(lab[u][c]), Q[c]))
        lines.append((names[u], ",".join(parts)))
    return tree_line, lines


def annotate(newick: str, char_mtrx: Dict[str, list], Q: List[dict], nu: float, phi: float,
             leaf_order: Sequence[str] = None, device="cuda", branch_lengths=None):
    """The exact-model E-step on the GPU at (the tree's branch lengths, or
    ``branch_lengths`` in the encoder's node order, nu, phi), then
    ``annotation_lines``."""
    et = encode_newick(newick, leaf_order)
    rows = [char_mtrx[et.labels[i]] for i in range(et.num_leaves)]
    ds = encode_dataset(char_matrix(rows, exact=True), Q, compat=False)
    d = et.branch_length if branch_lengths is None else np.asarray(branch_lengths, np.float64)
    b = DeviceBatch([ds], [et], [0], [d], [nu], [phi], compat=False,
                    want_post=True, device=device)
    b.e_step(want_post=True)
    cnt, _ = b.counts_from_partials()
    p0, p1 = b.posteriors(0)
    return annotation_lines(et, rows, Q, p0, p1, cnt[:, 1] + cnt[:, 2] + cnt[:, 4])
