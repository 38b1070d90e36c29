"""Host-side encoders: newick trees, character matrices and batch plans.

Thin wrappers over the C++ encoders of liblaml_gb300.so (laml_newick_*,
laml_dataset_*, laml_plan_*); all arrays are numpy.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _native as N

MISSING = -1
SILENCED = -2


@dataclass
class EncodedTree:
    """A tree in fastEM_solver.parse_tree numbering (fastEM_solver.py:46-146):
    leaves 0..n-1, internal nodes n..N-1 in treeswift preorder, children in
    networkx successor order."""
    num_nodes: int
    num_leaves: int
    parent: np.ndarray          # int32[N], -1 at the root
    child0: np.ndarray          # int32[N], -1 at leaves
    child1: np.ndarray
    branch_length: np.ndarray   # float64[N] (0 where absent)
    has_length: np.ndarray      # bool[N]
    labels: Optional[List[str]]

    @property
    def root(self) -> int:
        return int(np.flatnonzero(self.parent < 0)[0])


def encode_newick(newick: str, leaf_order: Optional[Sequence[str]] = None) -> EncodedTree:
    L = N.lib()
    nn, nl, lb = N.i32(), N.i32(), N.i64()
    s = newick.encode()
    N.check(L.laml_newick_size(s, C.byref(nn), C.byref(nl), C.byref(lb)))
    n_nodes = nn.value
    par = np.empty(n_nodes, np.int32)
    c0 = np.empty(n_nodes, np.int32)
    c1 = np.empty(n_nodes, np.int32)
    bl = np.empty(n_nodes, np.float64)
    has = np.empty(n_nodes, np.uint8)
    labels = C.create_string_buffer(int(lb.value) + 1)
    offs = np.empty(n_nodes, np.int64)
    if leaf_order is not None:
        arr = (C.c_char_p * len(leaf_order))(*[str(x).encode() for x in leaf_order])
        lo, nlo = arr, len(leaf_order)
    else:
        lo, nlo = None, 0
    N.check(L.laml_newick_encode(s, lo, nlo, N.ptr(par), N.ptr(c0), N.ptr(c1), N.ptr(bl),
                                 N.ptr(has), labels, N.ptr(offs)))
    raw = labels.raw
    labs = []
    for k in range(n_nodes):
        o = int(offs[k])
        e = raw.index(b"\0", o)
        labs.append(raw[o:e].decode())
    return EncodedTree(n_nodes, nl.value, par, c0, c1, bl, has.astype(bool), labs)


def encode_newick_batch(newicks: Sequence[str], leaf_order: Sequence[str],
                        n_threads: int = 0) -> List[EncodedTree]:
    """Many trees over one leaf set in one C call (laml_newick_encode_batch);
    the trees carry no labels (``labels`` is None)."""
    L = N.lib()
    T = len(newicks)
    arr = (C.c_char_p * T)(*[s.encode() for s in newicks])
    lo = (C.c_char_p * len(leaf_order))(*[str(x).encode() for x in leaf_order])
    tot = N.i64()
    N.check(L.laml_newick_batch_measure(T, arr, C.byref(tot)))
    m = tot.value
    par = np.empty(m, np.int32)
    c0 = np.empty(m, np.int32)
    c1 = np.empty(m, np.int32)
    bl = np.empty(m, np.float64)
    has = np.empty(m, np.uint8)
    off = np.empty(T + 1, np.int64)
    nl = np.empty(T, np.int32)
    N.check(L.laml_newick_encode_batch(T, arr, lo, len(leaf_order), n_threads, N.ptr(off),
                                       N.ptr(nl), N.ptr(par), N.ptr(c0), N.ptr(c1), N.ptr(bl),
                                       N.ptr(has)))
    out = []
    hb = has.astype(bool)
    for i in range(T):
        a, b = int(off[i]), int(off[i + 1])
        out.append(EncodedTree(b - a, int(nl[i]), par[a:b], c0[a:b], c1[a:b], bl[a:b], hb[a:b],
                               None))
    return out


def char_matrix(rows: Sequence[Sequence], exact: bool = False) -> np.ndarray:
    """Rows of {int, '?'} -> int32 codes: '?' (and anything non-numeric or
    negative) -> MISSING; an explicit -1 -> SILENCED when ``exact`` (EM_solver
    treats -1 as observed silencing, EM_solver.py:104-110), else MISSING
    (fastEM replaces '?' by -1, fastEM_solver.py:29)."""
    n = len(rows)
    K = len(rows[0]) if n else 0
    if any(len(r) != K for r in rows):
        raise ValueError("character matrix rows have different lengths")
    memo = {}

    def code(x):
        if isinstance(x, str):
            try:
                v = int(x)
            except ValueError:
                return MISSING
        else:
            v = int(x)
        return v if v >= 0 else (SILENCED if (exact and v == -1) else MISSING)

    def lookup(x):
        # rows repeat few distinct values: decode each once
        try:
            return memo[x]
        except KeyError:
            memo[x] = c = code(x)
            return c
        except TypeError:           # unhashable entry
            return code(x)

    flat = [lookup(x) for r in rows for x in r]
    return np.asarray(flat, np.int32).reshape(n, K)


def priors_csr(Q: Sequence[Dict], n_sites: int):
    """list of {state: prob} per site -> CSR (ptr, state, prob)."""
    if len(Q) != n_sites:
        raise ValueError(f"priors cover {len(Q)} sites, the matrix has {n_sites}")
    ptr = np.zeros(n_sites + 1, np.int32)
    st, pr = [], []
    for c, q in enumerate(Q):
        for k, v in q.items():
            st.append(int(k))
            pr.append(float(v))
        ptr[c + 1] = len(st)
    return ptr, np.asarray(st, np.int32), np.asarray(pr, np.float64)


@dataclass
class EncodedDataset:
    """Device site layout of one character matrix + priors (see
    laml_dataset_encode).  ``codes`` rows follow the tree's leaf order."""
    n_leaves: int
    n_sites: int
    n_sites_pad: int
    n_groups: int
    group_sites: int
    row_len: int
    max_states: int
    n_missing: int
    n_silenced: int
    codes: np.ndarray       # int16[n, Kpad]
    q: np.ndarray           # float32[row_len]
    site_perm: np.ndarray   # int32[Kpad]
    site_C: np.ndarray      # int32[Kpad]
    site_sumq: np.ndarray   # float32[Kpad]
    group_off: np.ndarray   # int32[NG]
    group_C: np.ndarray     # int32[NG]
    state_ptr: np.ndarray   # int32[K+1]
    state_map: np.ndarray   # int32[...]
    compat: bool


def encode_dataset(chars: np.ndarray, Q, compat: bool = True, group_sites: int = 8) -> EncodedDataset:
    """chars: int32[n, K] from char_matrix (leaf order); Q: per-site prior
    dicts or a (ptr, state, prob) CSR triple."""
    L = N.lib()
    chars = np.ascontiguousarray(chars, dtype=np.int32)
    n, K = chars.shape
    pp, ps, pq = Q if isinstance(Q, tuple) else priors_csr(Q, K)
    pp = np.ascontiguousarray(pp, np.int32)
    ps = np.ascontiguousarray(ps, np.int32)
    pq = np.ascontiguousarray(pq, np.float64)
    info = N.DatasetInfo()
    N.check(L.laml_dataset_measure(n, K, N.ptr(chars), N.ptr(pp), N.ptr(ps), N.ptr(pq),
                                   int(compat), group_sites, C.byref(info)))
    Kp, NG, R = info.n_sites_pad, info.n_groups, info.row_len
    codes = np.empty((n, Kp), np.int16)
    q = np.empty(R, np.float32)
    perm = np.empty(Kp, np.int32)
    sC = np.empty(Kp, np.int32)
    sq = np.empty(Kp, np.float32)
    goff = np.empty(NG, np.int32)
    gC = np.empty(NG, np.int32)
    sptr = np.empty(K + 1, np.int32)
    smap = np.empty(max(1, int(np.sum(chars > 0)) + K), np.int32)
    N.check(L.laml_dataset_encode(n, K, N.ptr(chars), N.ptr(pp), N.ptr(ps), N.ptr(pq),
                                  int(compat), group_sites, N.ptr(codes), N.ptr(q), N.ptr(perm),
                                  N.ptr(sC), N.ptr(sq), N.ptr(goff), N.ptr(gC), N.ptr(sptr),
                                  N.ptr(smap)))
    return EncodedDataset(n, K, Kp, NG, group_sites, R, info.max_states, info.n_missing,
                          info.n_silenced, codes, q, perm, sC, sq, goff, gC, sptr,
                          smap[:sptr[-1]].copy(), compat)


def nni_candidates(tree: EncodedTree, moves) -> List[EncodedTree]:
    """laml_nni_candidates: one EncodedTree per (u, u_child) move of
    ``tree`` (node ids), numbered as encoding the swapped tree's newick would
    number it; the candidates are views into shared arrays and carry no
    labels."""
    mv = np.ascontiguousarray(np.asarray(moves, np.int32).reshape(-1, 2))
    M, Nn = mv.shape[0], tree.num_nodes
    par = np.empty((M, Nn), np.int32)
    c0 = np.empty((M, Nn), np.int32)
    c1 = np.empty((M, Nn), np.int32)
    bl = np.empty((M, Nn), np.float64)
    has = np.empty((M, Nn), np.uint8)
    src = [np.ascontiguousarray(a, t) for a, t in
           ((tree.parent, np.int32), (tree.child0, np.int32), (tree.child1, np.int32),
            (tree.branch_length, np.float64), (tree.has_length, np.uint8))]
    N.check(N.lib().laml_nni_candidates(Nn, tree.num_leaves, *[a.ctypes.data for a in src], M,
                                        mv.ctypes.data, 0, par.ctypes.data, c0.ctypes.data,
                                        c1.ctypes.data, bl.ctypes.data, has.ctypes.data))
    hb = has.astype(bool)
    return [EncodedTree(Nn, tree.num_leaves, par[m], c0[m], c1[m], bl[m], hb[m], None)
            for m in range(M)]


def plan_batch(trees: Sequence[EncodedTree], tree_ds: Sequence[int],
               datasets: Sequence[EncodedDataset], host_desc: bool = True,
               items: bool = True):
    """Level schedule + buffer offsets of a batch (laml_plan_*).  Returns
    (sizes: dict, arrays: dict of numpy arrays).  With ``host_desc`` False
    the item and group descriptors are left out (laml_plan_descriptors
    builds them on the device).  With ``items`` False (device descriptors,
    every dataset with the same group count) the (node, group) item lists
    are replaced by the level node lists ``in_lnodes`` / ``out_lnodes``,
    which laml_plan_descriptors expands on the device."""
    L = N.lib()
    T = len(trees)
    tn = np.asarray([t.num_nodes for t in trees], np.int32)
    tl = np.asarray([t.num_leaves for t in trees], np.int32)
    td = np.asarray(tree_ds, np.int32)
    c0 = np.concatenate([t.child0 for t in trees]).astype(np.int32)
    c1 = np.concatenate([t.child1 for t in trees]).astype(np.int32)
    dg = np.asarray([d.n_groups for d in datasets], np.int32)
    dk = np.asarray([d.n_sites_pad for d in datasets], np.int32)
    dr = np.asarray([d.row_len for d in datasets], np.int64)
    gbase = np.zeros(len(datasets), np.int32)
    gbase[1:] = np.cumsum(dg)[:-1]
    gC = np.concatenate([d.group_C for d in datasets]).astype(np.int32)
    dK = np.asarray([d.n_sites for d in datasets], np.int32)
    dn = np.asarray([d.n_leaves for d in datasets], np.int32)
    goff = np.concatenate([d.group_off for d in datasets]).astype(np.int32)
    pin = N.PlanInput(T, N.ptr(tn), N.ptr(tl), N.ptr(td), N.ptr(c0), N.ptr(c1), len(datasets),
                      N.ptr(dg), N.ptr(dk), N.ptr(dr), N.ptr(gbase), N.ptr(gC), N.ptr(dK),
                      N.ptr(dn), N.ptr(goff))
    sz = N.PlanSizes()
    N.check(L.laml_plan_measure(C.byref(pin), C.byref(sz)))
    nn = sz.n_nodes
    arr = {
        "tr_node_base": np.empty(T, np.int32), "tr_root": np.empty(T, np.int32),
        "tr_quirk": np.empty(T, np.int32), "tr_site_base": np.empty(T, np.int64),
        "tr_cnt_base": np.empty(T, np.int64), "tr_post_base": np.empty(T, np.int64),
        "nd_tree": np.empty(nn, np.int32), "nd_c0": np.empty(nn, np.int32),
        "nd_c1": np.empty(nn, np.int32), "nd_parent": np.empty(nn, np.int32),
        "nd_sib": np.empty(nn, np.int32), "nd_leafrow": np.empty(nn, np.int32),
        "nd_prow": np.empty(nn, np.int64), "nd_srow": np.empty(nn, np.int64),
        "in_level_off": np.empty(sz.n_in_levels + 1, np.int32),
        "out_level_off": np.empty(sz.n_out_levels + 1, np.int32),
        "root_items": np.empty(2 * max(1, sz.n_root_items), np.int32),
    }
    if not items and (host_desc or len({d.n_groups for d in datasets}) != 1):
        items = True   # host descriptors, or datasets of different group counts
    if items:
        arr["in_items"] = np.empty(2 * max(1, sz.n_in_items), np.int32)
        arr["out_items"] = np.empty(2 * max(1, sz.n_out_items), np.int32)
    else:
        n_int = int(np.sum(tn) - np.sum(tl))
        arr["in_lnodes"] = np.empty(max(1, n_int), np.int32)
        arr["out_lnodes"] = np.empty(max(1, n_int), np.int32)
    if host_desc:
        arr["in_desc"] = np.empty(12 * max(1, sz.n_in_items), np.int32)
        arr["out_desc"] = np.empty(12 * max(1, sz.n_out_items), np.int32)
        arr["grp_desc"] = np.empty(8 * max(1, sz.n_groups_total), np.int32)
    pout = N.PlanOutput(*[N.ptr(arr[k]) if k in arr else None for k in N.PLAN_OUT_FIELDS])
    N.check(L.laml_plan_fill(C.byref(pin), C.byref(pout)))
    sizes = {k: getattr(sz, k) for k, _ in N.PlanSizes._fields_}
    arr["group_base"] = gbase
    return sizes, arr
