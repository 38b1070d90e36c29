"""FP64 CPU oracle for LAML's PMM likelihood / EM hot path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: it may be imported by
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / reference
leg of ``bench.py`` and nowhere else.  The product path (``laml_gb300``) never
imports it and never falls back to it.

It restates, in NumPy float64 and in log space, with the reference's dense
padded layout (sites x states, states ordered 0, 1..k, silenced):

* treeswift newick parsing and the fastEM node numbering
  (laml_libs/fastEM_solver.py:46-146; treeswift>=1.1.39 stack-based preorder)
* character / prior recoding (fast_em/phylogeny.py:48-114)
* leaf init, edge-inside, inside, outside, responsibilities, E-step
  (fast_em/calculations.py:11-577)
* the fastEM M-step objective (fast_em/laml.py:49-78) maximised by
  coordinate ascent, and the fastEM EM loop (fast_em/laml.py:112-194)
* the exact-model EM of laml_libs/EM_solver.py:91-512 (normalised priors,
  no EPS floors, '?' vs explicit silencing, S0..S4 normalisation, bounded
  branch-length and nu solves, closed-form phi), restated in the full-state
  form: the alpha-clade bookkeeping of ML_solver.az_partition
  (ML_solver.py:125-154) is a compression of exactly these sums.
* posteriors and the annotation strings (laml_libs/runner.py:367-435)

Two model modes share every function:

``compat=True``  -- fast_em semantics: EPS=1e-6 floors on the leaf emission
                    and on 1-e^{-d}, 1-e^{-nu d}; priors are the raw priors of
                    the *observed* states (no renormalisation); '?' and -1 are
                    both "missing"; the root's E-step row indexes node N-1
                    (parent_sibling[root] = (-1, -1), fast_em/laml.py:244-246).
``compat=False`` -- EM_solver semantics: priors normalised per site, the mass
                    of unobserved mutated states kept as one lumped state,
                    no floors, '?' = missing and -1 = silenced, and the root's
                    counts taken from a progenitor in state 0.

Parity pins (tests/test_oracle_golden.py): the 3-leaf known-answer nllh values
of laml_unit_tests/unit_tests_EMSolver.py test_1..20, 46 and
unit_tests_MLSolver.py; the reduced-tree outside identity of
unit_tests_EMSolver.py:247-303 (tests 21-45, including the 150x60 test1 data);
the EM fixed point of unit_tests_EMSolver.py:535-602 (test4 data, nllh
1007.009158767873 rel 1e-4, phi = nu = 0); and compat == exact whenever the
observed priors sum to one and EPS -> 0.  The fastEM M-step in the reference is
100 optax L-BFGS steps, which are not reproducible without optax: this oracle
maximises the same objective to its stationary point instead, so parity with
the reference's own fastEM iterates is unpinned and is stated at the EM fixed
point (unit_tests_fastEMSolver.py:40-44, |d nllh| < 10).
"""
from __future__ import annotations

import math
import random as _random
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

EPS = 1e-6                 # fast_em/calculations.py:9
CALC_EPS = 1e-10           # fast_em/laml.py:47
EM_STOP_COMPAT = 1e-5      # fast_em/laml.py:46
CONV_EPS_EXACT = 1e-8      # laml_libs/core_constants.py:5
DMIN, DMAX = 0.005, 10.0   # laml_libs/core_constants.py:7-8
EPS_S = 1e-6               # EM_solver.Mstep eps_s (EM_solver.py:307)
EPS_NU = 1e-5              # EM_solver.Mstep eps_nu (EM_solver.py:307)
NEG_INF = -np.inf
MISSING = -1               # '?'
SILENCED = -2              # explicit -1 in the exact model


# ----------------------------------------------------------------------------
# newick parsing with treeswift traversal semantics
# ----------------------------------------------------------------------------
class Node:
    __slots__ = ("label", "length", "children", "parent")

    def __init__(self):
        self.label: Optional[str] = None
        self.length: Optional[float] = None
        self.children: List["Node"] = []
        self.parent: Optional["Node"] = None

    def is_leaf(self):
        return len(self.children) == 0


def read_newick(s: str) -> Node:
    """Parse a newick string (labels, ':length', nested parentheses)."""
    s = s.strip()
    i = 0
    n = len(s)
    root = Node()
    cur = root
    stack: List[Node] = []

    def read_token(j):
        k = j
        while k < n and s[k] not in ",():;[":
            k += 1
        return s[j:k].strip(), k

    while i < n:
        ch = s[i]
        if ch == "(":
            child = Node()
            child.parent = cur
            cur.children.append(child)
            stack.append(cur)
            cur = child
            i += 1
        elif ch == ",":
            parent = stack[-1]
            child = Node()
            child.parent = parent
            parent.children.append(child)
            cur = child
            i += 1
        elif ch == ")":
            cur = stack.pop()
            i += 1
        elif ch == ":":
            tok, i = read_token(i + 1)
            cur.length = float(tok)
        elif ch == ";":
            break
        elif ch == "[":
            j = s.index("]", i)
            i = j + 1
        elif ch.isspace():
            i += 1
        else:
            tok, i = read_token(i)
            if tok:
                cur.label = tok
    return root


def write_newick(root: Node) -> str:
    """Serialise a parsed tree back to newick (labels and lengths)."""
    def rec(v):
        s = ""
        if v.children:
            s = "(" + ",".join(rec(c) for c in v.children) + ")"
        if v.label is not None:
            s += v.label
        if v.length is not None:
            s += ":" + repr(float(v.length))
        return s
    return rec(root) + ";"


def preorder(root: Node):
    """treeswift Node.traverse_preorder: a stack, children pushed in order."""
    st = [root]
    while st:
        v = st.pop()
        yield v
        st.extend(v.children)


def postorder(root: Node):
    """treeswift Node.traverse_postorder (children visited in order)."""
    s1, s2 = [root], []
    while s1:
        v = s1.pop()
        s2.append(v)
        s1.extend(v.children)
    while s2:
        yield s2.pop()


@dataclass
class ParsedTree:
    labels: List[str]              # relabeling_vector
    num_leaves: int
    parent: np.ndarray             # int64[N], -1 for the root
    children: List[List[int]]      # networkx successor order
    branch_lengths: np.ndarray     # float64[N]
    has_length: np.ndarray         # bool[N]
    root: int


def parse_tree(newick: str, ordered_leaf_labels: Optional[Sequence[str]] = None,
               rng=None) -> ParsedTree:
    """fastEM_solver.parse_tree (fastEM_solver.py:46-146).

    Nodes enter the graph in treeswift preorder (so networkx successors are
    the newick children in reverse order); a unifurcating root is dropped;
    leaves get 0..n-1 (in ``ordered_leaf_labels`` order when given, else
    preorder), internal nodes n..N-1 in preorder.  Missing lengths draw
    ``rng.uniform(0.01, 0.5)`` in that order (lines 95, 110, 126)."""
    rng = rng if rng is not None else _random
    root = read_newick(newick)
    order = list(preorder(root))
    labels = []
    for idx, v in enumerate(order):
        if v.label is None:
            v.label = f"node_{idx}"
        labels.append(v.label)
    succ: Dict[str, List[str]] = {v.label: [] for v in order}
    pred: Dict[str, Optional[str]] = {v.label: None for v in order}
    length = {v.label: v.length for v in order}
    nodes = [v.label for v in order]
    for v in order:
        if v.parent is not None:
            succ[v.parent.label].append(v.label)
            pred[v.label] = v.parent.label
    r = nodes[0]
    if len(succ[r]) == 1:
        c = succ[r][0]
        pred[c] = None
        nodes = nodes[1:]
        del succ[r]
    leaves_in_order = [x for x in nodes if len(succ[x]) == 0]
    if ordered_leaf_labels is not None:
        leafset = set(leaves_in_order)
        leaf_seq = [x for x in ordered_leaf_labels if x in leafset]
    else:
        leaf_seq = leaves_in_order
    relabel: Dict[str, int] = {}
    bl, has = [], []
    for x in leaf_seq:
        relabel[x] = len(relabel)
        b = length[x]
        has.append(b is not None)
        bl.append(b if b is not None else rng.uniform(0.01, 0.5))
    n = len(relabel)
    for x in nodes:
        if len(succ[x]) > 0:
            relabel[x] = len(relabel)
            b = length[x]
            has.append(b is not None)
            bl.append(b if b is not None else rng.uniform(0.01, 0.5))
    N = len(relabel)
    vec = sorted(relabel, key=lambda z: relabel[z])
    parent = np.full(N, -1, dtype=np.int64)
    children: List[List[int]] = [[] for _ in range(N)]
    for x in nodes:
        i = relabel[x]
        for c in succ[x]:
            children[i].append(relabel[c])
            parent[relabel[c]] = i
    roots = [i for i in range(N) if parent[i] < 0]
    assert len(roots) == 1
    return ParsedTree(vec, n, parent, children, np.asarray(bl, dtype=np.float64),
                      np.asarray(has, dtype=bool), roots[0])


# ----------------------------------------------------------------------------
# recoding (fast_em/phylogeny.py:48-114) and the exact-model prior table
# ----------------------------------------------------------------------------
@dataclass
class Encoded:
    chars: np.ndarray          # int64[n, K]: 0, 1..k_c, MISSING, SILENCED
    q: np.ndarray              # float64[K, Chat-2] (zero padded)
    k: np.ndarray              # observed mutated states per site (+1 lumped in exact)
    state_maps: List[List]     # recoded index-1 -> original state
    compat: bool


def recode(rows: Sequence[Sequence], Q: Sequence[Dict], compat: bool = True) -> Encoded:
    """rows[i][c] in {int, '?'} in leaf order; Q[c] = {state: prior}.

    compat: '?' and -1 -> MISSING; priors are the raw float32 priors of the
    observed states (phylogeny.py:80-94).  exact: '?' -> MISSING, -1 ->
    SILENCED, priors normalised over the whole dict (ML_solver.py:69-74) with
    the remaining mass as one extra state that no leaf shows."""
    n = len(rows)
    K = len(rows[0]) if n else 0
    raw = np.zeros((n, K), dtype=np.int64)
    for i, r in enumerate(rows):
        for c, x in enumerate(r):
            if x == "?" or x == "-":
                raw[i, c] = MISSING
            else:
                xi = int(x)
                if xi == -1:
                    raw[i, c] = MISSING if compat else SILENCED
                elif xi < 0:
                    raw[i, c] = MISSING
                else:
                    raw[i, c] = xi
    chars = raw.copy()
    ks, maps, qcols = [], [], []
    for c in range(K):
        valid = sorted(set(int(x) for x in raw[:, c]) - {MISSING, SILENCED, 0})
        mp = {o: j + 1 for j, o in enumerate(valid)}
        for i in range(n):
            if raw[i, c] > 0:
                chars[i, c] = mp[int(raw[i, c])]
        Qc = Q[c]
        qd = {}
        for key, val in Qc.items():
            qd[int(key)] = float(val)
        if compat:
            col = []
            for o in valid:
                if o not in qd:
                    raise KeyError(f"missing mutation prior for character {c}, state {o}")
                col.append(float(np.float32(qd[o])))
        else:
            tot = sum(qd.values())
            col = []
            for o in valid:
                if o not in qd:
                    raise KeyError(f"missing mutation prior for character {c}, state {o}")
                col.append(qd[o] / tot)
            col.append(max(0.0, 1.0 - sum(col)))   # lumped unobserved states
        ks.append(len(col))
        maps.append(valid)
        qcols.append(col)
    kmax = max(ks) if ks else 0
    q = np.zeros((K, kmax))
    for c in range(K):
        q[c, :len(qcols[c])] = qcols[c]
    return Encoded(chars, q, np.asarray(ks), maps, compat)


# ----------------------------------------------------------------------------
# the numeric core (fast_em/calculations.py), log space, float64
# ----------------------------------------------------------------------------
def lse(x, axis):
    m = np.max(x, axis=axis, keepdims=True)
    m0 = np.where(np.isfinite(m), m, 0.0)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        r = np.log(np.sum(np.exp(x - m0), axis=axis, keepdims=True)) + m0
    r = np.where(np.isneginf(m), NEG_INF, r)
    return np.squeeze(r, axis=axis)


def _log(x):
    with np.errstate(divide="ignore"):
        return np.log(x)


def branch_terms(d, nu, eps):
    """t1, t2, t3, alpha0 (calculations.py:153-157): t2 = log(1-e^{-nu d}) and
    t3 = log(1-e^{-d}) floored at log(eps) below eps (no floor if eps == 0)."""
    d = np.asarray(d, dtype=np.float64)
    nd = d * nu
    lfe = math.log(eps) if eps > 0 else NEG_INF
    with np.errstate(divide="ignore", invalid="ignore"):
        t2 = np.where(nd < eps, lfe, _log(-np.expm1(-nd)))
        t3 = np.where(d < eps, lfe, _log(-np.expm1(-d)))
    return -nd, t2, t3, -d * (1.0 + nu)


def leaf_inside(chars, phi, C, eps):
    """initialize_leaf_inside_log_likelihoods (calculations.py:278-334); the
    exact model adds SILENCED leaves (EM_solver.py:104-110)."""
    a = np.arange(C)[None, None, :]
    c = chars[:, :, None]
    s = C - 1
    miss = c == MISSING
    sil = c == SILENCED
    conds = [(a == s) & (miss | sil), (a == s) & ~(miss | sil), a == c, miss]
    ch = [max(1.0, eps), max(0.0, eps), max(1.0 - phi, eps), max(phi, eps)]
    return _log(np.select(conds, ch, default=0.0))


def edge_inside(x, logq, t1, t2, t3, a0):
    """compute_Q_transpose_v_product (calculations.py:47-91); x is (K, C)."""
    K, C = x.shape
    out = np.empty_like(x)
    summ = np.empty_like(x)
    summ[:, 0] = a0
    summ[:, 1:-1] = t1 + logq + t3
    summ[:, -1] = t2
    out[:, 0] = lse(summ + x, axis=1)
    out[:, 1:-1] = np.logaddexp(t1 + x[:, 1:-1], t2 + x[:, -1:])
    out[:, -1] = x[:, -1]
    return out


def q_v_product(x, logq, t1, t2, t3, a0):
    """compute_Q_v_product (calculations.py:11-45)."""
    out = np.empty_like(x)
    out[:, 0] = a0 + x[:, 0]
    out[:, -1] = np.logaddexp(t2 + lse(x[:, :-1], axis=1), x[:, -1])
    out[:, 1:-1] = np.logaddexp(logq + t1 + t3 + x[:, 0:1], t1 + x[:, 1:-1])
    return out


@dataclass
class Problem:
    tree: ParsedTree
    enc: Encoded
    compat: bool = True

    @property
    def C(self):
        return self.enc.q.shape[1] + 2

    @property
    def eps(self):
        return EPS if self.compat else 0.0

    @property
    def logq(self):
        return _log(self.enc.q)

    def sibling(self, v):
        p = self.tree.parent[v]
        if p < 0:
            return -1
        sib = [c for c in self.tree.children[p] if c != v]
        return sib[0]


def inside(prob: Problem, d, nu, phi):
    """Leaf init + inside pass + root edge (calculations.py:193-334).
    Returns (inside (N, K, C) log, root_llh (K,), terms)."""
    tr, enc = prob.tree, prob.enc
    N, n, K, C = len(tr.parent), tr.num_leaves, enc.chars.shape[1], prob.C
    t = branch_terms(d, nu, prob.eps)
    logq = prob.logq
    ins = np.full((N, K, C), math.log(EPS) if prob.compat else NEG_INF)
    ins[:n] = leaf_inside(enc.chars, phi, C, prob.eps)
    for u in _postorder_ids(tr):
        if u < n:
            continue
        acc = np.zeros((K, C))
        for v in tr.children[u]:
            acc = acc + edge_inside(ins[v], logq, t[0][v], t[1][v], t[2][v], t[3][v])
        ins[u] = acc
    r = tr.root
    root_edge = edge_inside(ins[r], logq, t[0][r], t[1][r], t[2][r], t[3][r])
    return ins, root_edge[:, 0], t


def _postorder_ids(tr: ParsedTree):
    out, st = [], [(tr.root, False)]
    while st:
        u, done = st.pop()
        if done:
            out.append(u)
            continue
        st.append((u, True))
        for c in reversed(tr.children[u]):
            st.append((c, False))
    return out


def _preorder_ids(tr: ParsedTree):
    out, st = [], [tr.root]
    while st:
        u = st.pop()
        out.append(u)
        st.extend(reversed(tr.children[u]))
    return out


def log_likelihood(prob: Problem, d, nu, phi):
    """compute_log_likelihood (calculations.py:456-504): sum over sites of the
    root edge from a progenitor in state 0.  Returns (total, per_site)."""
    _, root_llh, _ = inside(prob, d, nu, phi)
    return float(np.sum(root_llh)), root_llh


@dataclass
class EStep:
    llh: float
    llh_site: np.ndarray      # (K,)
    counts: np.ndarray        # (N, 6): C00 C0a C0s Caa Cas Css summed over sites
    leaf_resp: np.ndarray     # (n,)  P(leaf silenced | D) summed over sites
    inside: np.ndarray
    outside: np.ndarray
    edge_in: np.ndarray
    post0: np.ndarray         # (N, K) log P(v = 0 | D)
    post1: np.ndarray         # (N, K) log P(v = silenced | D)


FLT_MIN = 1.1754943508222875e-38


def _ftz(x, compat):
    """fast_em exponentiates its log-responsibilities in float32 with
    denormals flushed (calculations.py:576-577): in the compat model a
    per-site term below the smallest normal float is zero.  The exact model
    (EM_solver, float64) keeps them."""
    return np.where(x < FLT_MIN, 0.0, x) if compat else x


def e_step(prob: Problem, d, nu, phi) -> EStep:
    """compute_E_step (calculations.py:506-577) plus the posteriors of
    EM_solver.Estep_posterior (EM_solver.py:247-300)."""
    tr = prob.tree
    N, n = len(tr.parent), tr.num_leaves
    ins, L, t = inside(prob, d, nu, phi)
    K, C = ins.shape[1], ins.shape[2]
    logq = prob.logq
    ein = np.empty_like(ins)
    for v in range(N):
        ein[v] = edge_inside(ins[v], logq, t[0][v], t[1][v], t[2][v], t[3][v])
    out = np.zeros_like(ins)
    r = tr.root
    out[r, :, 0] = t[3][r]
    out[r, :, -1] = t[1][r]
    out[r, :, 1:-1] = t[0][r] + logq + t[2][r]
    for v in _preorder_ids(tr):
        if v == r:
            continue
        u, w = tr.parent[v], prob.sibling(v)
        out[v] = q_v_product(out[u] + ein[w], logq, t[0][v], t[1][v], t[2][v], t[3][v])
    counts = np.zeros((N, 6))
    lr = L[:, None]
    for v in range(N):
        if v == r:
            if prob.compat:   # parent_sibling[root] = (-1, -1) -> node N-1
                x = out[N - 1] + ein[N - 1]
            else:             # progenitor in state 0
                x = np.full((K, C), NEG_INF)
                x[:, 0] = 0.0
        else:
            x = out[tr.parent[v]] + ein[prob.sibling(v)]
        iv = ins[v]
        t1, t2, t3, a0 = t[0][v], t[1][v], t[2][v], t[3][v]
        c00 = x[:, 0] + iv[:, 0] + a0 - L
        c0a = lse(x[:, 0:1] + iv[:, 1:-1] + t1 + logq + t3 - lr, axis=1)
        c0s = x[:, 0] + iv[:, -1] + t2 - L
        caa = lse(x[:, 1:-1] + iv[:, 1:-1] + t1 - lr, axis=1)
        cas = lse(x[:, 1:-1] + iv[:, -1:] + t2 - lr, axis=1)
        css = x[:, -1] + iv[:, -1] - L
        with np.errstate(over="ignore"):
            counts[v] = _ftz(np.exp(np.stack([c00, c0a, c0s, caa, cas, css])),
                             prob.compat).sum(axis=1)
    with np.errstate(over="ignore"):
        leaf_resp = _ftz(np.exp(ins[:n, :, -1] + out[:n, :, -1] - L[None, :]),
                         prob.compat).sum(axis=1)
    post0 = ins[:, :, 0] + out[:, :, 0] - L[None, :]
    post1 = ins[:, :, -1] + out[:, :, -1] - L[None, :]
    return EStep(float(np.sum(L)), L, counts, leaf_resp, ins, out, ein, post0, post1)


# ----------------------------------------------------------------------------
# M-steps
# ----------------------------------------------------------------------------
def _log1mexp(x):
    x = np.asarray(x, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(x > math.log(2.0), np.log1p(-np.exp(-x)), np.log(-np.expm1(-x)))


def _inv_expm1(x):
    """1 / (e^x - 1) for x >= 0 (inf at 0)."""
    with np.errstate(divide="ignore", over="ignore"):
        return 1.0 / np.expm1(x)


def mstep_objective_compat(counts, leaf_resp_total, R, M, d, nu, phi):
    """-(M_step_loss_fn) of fast_em/laml.py:62-78 (to be maximised)."""
    d = np.clip(d, CALC_EPS, 1.0 / CALC_EPS)
    nu = min(max(nu, CALC_EPS), 1 - CALC_EPS)
    phi = min(max(phi, CALC_EPS), 1 - CALC_EPS)
    e = counts
    c1 = -e[:, 0] * d * (1.0 + nu)
    c2 = e[:, 1] * (_log1mexp(d) - d * nu)
    c3 = e[:, 2] * _log1mexp(d * nu)
    c4 = -e[:, 3] * d * nu
    c5 = e[:, 4] * _log1mexp(d * nu)
    c6 = R * math.log(1 - phi) + (M - leaf_resp_total) * math.log(phi)
    return float(np.sum(c1 + c2 + c3 + c4 + c5) + c6)


def _bisect_decreasing(fprime, lo, hi, iters=200):
    """Root of a decreasing vector function on [lo, hi] in log space; clips to
    the end points when the sign does not change."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    flo = fprime(lo)
    fhi = fprime(hi)
    a, b = np.log(lo), np.log(hi)
    for _ in range(iters):
        m = 0.5 * (a + b)
        fm = fprime(np.exp(m))
        pos = fm > 0
        a = np.where(pos, m, a)
        b = np.where(pos, b, m)
    x = np.exp(0.5 * (a + b))
    x = np.where(flo <= 0, lo, x)
    x = np.where(fhi >= 0, hi, x)
    return x


MSTEP_ROUNDS = 4


def mstep_compat(counts, leaf_resp_total, R, M, d, nu, phi, branch_mask, fix_nu, fix_phi,
                 rounds=MSTEP_ROUNDS):
    """Maximise the fast_em M-step objective (laml.py:62-78) over
    (d, nu, phi) by coordinate ascent: closed-form phi, per-branch 1-D solves
    of d given nu, a 1-D solve of nu given d.  d in [1e-10, 1e10] and
    nu, phi in [1e-10, 1-1e-10] (exp_safe / sigmoid_clamped)."""
    d = np.asarray(d, dtype=np.float64).copy()
    e = counts
    if not fix_phi:
        B = M - leaf_resp_total
        phi = B / (R + B) if (R + B) > 0 else phi
        phi = min(max(phi, CALC_EPS), 1 - CALC_EPS)
    mask = np.asarray(branch_mask, dtype=bool)
    b = e[:, 1]
    c = e[:, 2] + e[:, 4]
    for _ in range(rounds):
        if mask.any():
            a = e[:, 0] * (1.0 + nu) + (e[:, 1] + e[:, 3]) * nu

            def fp(x):
                return -a + b * _inv_expm1(x) + c * nu * _inv_expm1(nu * x)

            lo = np.full(len(d), CALC_EPS)
            hi = np.full(len(d), 1.0 / CALC_EPS)
            dn = _bisect_decreasing(fp, lo, hi)
            # a branch without expected counts has a zero gradient: the
            # L-BFGS of laml.py:94-119 leaves it unchanged
            flat = (a == 0) & (b == 0) & (c == 0)
            d = np.where(mask & ~flat, dn, d)
        if not fix_nu:
            A = float(np.sum((e[:, 0] + e[:, 1] + e[:, 3]) * d))

            def gp(x):
                x = float(x)
                return -A + float(np.sum(c * d * _inv_expm1(x * d)))

            nu = float(_bisect_decreasing(np.vectorize(gp), np.array(CALC_EPS),
                                          np.array(1 - CALC_EPS), iters=200))
    return d, nu, phi


def mstep_exact(counts, post1_leaf_missing_sum, R, d, nu, phi, branch_mask, K, ncells,
                opt_phi=True, opt_nu=True, ultra_tree: Optional[ParsedTree] = None,
                ultra_constraints=None):
    """EM_solver.Mstep (EM_solver.py:307-459) without MOSEK: closed-form phi
    (318-326), per-branch S normalisation (339-348), d in [dmin, dmax] given
    the old nu (349-366) and nu in [0, 1] given the new d (392-407), each a
    1-D concave problem solved by bisection.  ``counts`` are the full-state
    C00..Cas = S0..S4.  ``post1_leaf_missing_sum`` is sum over '?' leaf
    entries of P(leaf silenced | D).  With ``ultra_tree`` the branch lengths
    are solved jointly under that tree's ultrametric equalities
    (ultrametric_d) and a fourth item reports whether that solve succeeded
    (False: EM_solver's "d_infeasible")."""
    d = np.asarray(d, dtype=np.float64).copy()
    nmiss = post1_leaf_missing_sum[1]
    if opt_phi:
        Rt = nmiss - post1_leaf_missing_sum[0]
        phi_star = Rt / (R + Rt)
        if abs(phi_star) < 1.0 / (K * ncells):
            phi_star = 0.0
    else:
        phi_star = phi
    mask = np.asarray(branch_mask, dtype=bool)
    S = np.maximum(counts[:, :5], EPS_S)
    S = S / S.sum(axis=1, keepdims=True) * K
    S0, S1, S2, S3, S4 = (S[:, i] for i in range(5))
    Sm = S[mask]
    use_s = nu > EPS_NU

    a = (nu + 1) * S0 + nu * S1 + nu * S3
    c = (S2 + S4) if use_s else np.zeros_like(S2)

    def fp(x):
        return -a + S1 * _inv_expm1(x) + c * nu * _inv_expm1(nu * x)

    ultra = ultra_tree is not None or ultra_constraints is not None
    if ultra:
        d, ok = ultrametric_d(S, nu, d, mask, ultra_tree, ultra_constraints)
        if not ok:
            return d, nu, phi, False
    else:
        dn = _bisect_decreasing(fp, np.full(len(d), DMIN), np.full(len(d), DMAX))
        d = np.where(mask, dn, d)
    if opt_nu:
        dm = d[mask]
        A = float(np.sum((Sm[:, 0] + Sm[:, 1] + Sm[:, 3]) * dm))
        cc = Sm[:, 2] + Sm[:, 4]

        def gp(x):
            return -A + float(np.sum(cc * dm * _inv_expm1(float(x) * dm)))

        g1 = gp(1.0)
        if g1 >= 0:
            nu = 1.0
        elif cc.sum() <= 0:
            nu = 0.0
        else:
            nu = float(_bisect_decreasing(np.vectorize(gp), np.array(1e-300), np.array(1.0),
                                          iters=300))
    if ultra:
        return d, nu, phi_star, True
    return d, nu, phi_star


def ultrametric_constraints(tree: ParsedTree, mask, d):
    """EM_solver.ultrametric_constr (EM_solver.py:53-89) for one tree: rows M
    and right-hand sides b of ``M @ d[free] = b``, columns the optimised
    branches (``mask``) in treeswift postorder.  A node's path vector is its
    own branch plus its first child's (treeswift's first child: the last
    networkx successor); each internal node equates its two children's
    paths, fixed branches entering as constants, and a row whose vector is
    zero or repeats an earlier row (or its negation) is dropped, as there."""
    post = treeswift_postorder_ids(tree)
    mask = np.asarray(mask, bool)
    free = [x for x in post if mask[x]]
    col = {x: i for i, x in enumerate(free)}
    n = len(free)
    vec, const, rows = {}, {}, {}
    for x in post:
        ch = tree.children[x]
        if not ch:
            v = np.zeros(n)
            c = 0.0 if mask[x] else float(d[x])
        else:
            c1, c2 = ch[-1], ch[0]
            m = vec[c1] - vec[c2]
            if np.any(m != 0):
                key, neg = tuple(m), tuple(-m)
                if key not in rows and neg not in rows:
                    rows[key] = const[c2] - const[c1]
            v = vec[c1].copy()
            c = const[c1] + (0.0 if mask[x] else float(d[x]))
        if mask[x]:
            v[col[x]] = 1.0
        vec[x], const[x] = v, c
    M = np.array([list(k) for k in rows], dtype=np.float64).reshape(len(rows), n)
    b = np.array(list(rows.values()), dtype=np.float64)
    return M, b, np.array(free, dtype=np.int64)


def ultrametric_constraints_forest(trees: Sequence[ParsedTree], masks, ds):
    """EM_solver.ultrametric_constr (EM_solver.py:53-89) for several trees:
    each tree's rows, columns the optimised branches of all trees (tree by
    tree, treeswift postorder), then one row per further tree equating its
    root's path (its own branch included) with the first tree's
    (EM_solver.py:81-84).  ``free`` indexes the trees' concatenated branch
    vectors."""
    vecs, consts, rows = [], [], {}
    cols, off, ncol = [], 0, 0
    per = []
    for tr, mask, d in zip(trees, masks, ds):
        post = treeswift_postorder_ids(tr)
        mask = np.asarray(mask, bool)
        free = [x for x in post if mask[x]]
        per.append((tr, post, mask, d, free, ncol))
        cols += [off + x for x in free]
        ncol += len(free)
        off += len(tr.parent)
    roots = []
    for tr, post, mask, d, free, c0 in per:
        col = {x: c0 + i for i, x in enumerate(free)}
        vec, const = {}, {}
        for x in post:
            ch = tr.children[x]
            if not ch:
                v = np.zeros(ncol)
                c = 0.0 if mask[x] else float(d[x])
            else:
                a, b_ = ch[-1], ch[0]
                m = vec[a] - vec[b_]
                if np.any(m != 0):
                    key, neg = tuple(m), tuple(-m)
                    if key not in rows and neg not in rows:
                        rows[key] = const[b_] - const[a]
                v = vec[a].copy()
                c = const[a] + (0.0 if mask[x] else float(d[x]))
            if mask[x]:
                v[col[x]] = 1.0
            vec[x], const[x] = v, c
        roots.append((vec[tr.root], const[tr.root]))
    for v, c in roots[1:]:
        rows[tuple(roots[0][0] - v)] = c - roots[0][1]
    M = np.array([list(k) for k in rows], dtype=np.float64).reshape(len(rows), ncol)
    b = np.array(list(rows.values()), dtype=np.float64)
    return M, b, np.array(cols, dtype=np.int64)


def ultrametric_d(S, nu, d, mask, tree: Optional[ParsedTree], constraints=None):
    """The branch-length part of EM_solver.Mstep with ultra_constr_cache
    (EM_solver.py:349-366): maximise over the optimised branches
    sum -a d + S1 log(1-e^{-d}) + c log(1-e^{-nu d}) with d in [dmin, dmax]
    and ``M d = b`` (ultrametric_constraints).  The reference hands this to
    MOSEK (absent here).  This restatement: a strictly feasible start from a
    linear program (maximise the smallest slack to the bounds on the affine
    set), then a dense log-barrier Newton method in the null space of M
    (FP64, duality gap below 1e-11 relative).  Returns (d, ok); ok is False
    when the constraints leave no interior point (EM_solver's
    "d_infeasible")."""
    from scipy import linalg, optimize

    S0, S1, S2, S3, S4 = (S[:, i] for i in range(5))
    use_s = nu > EPS_NU
    M, rhs, free = constraints if constraints is not None else \
        ultrametric_constraints(tree, mask, d)
    n = len(free)
    out = np.asarray(d, np.float64).copy()
    if n == 0:
        return out, True
    a = ((nu + 1) * S0 + nu * S1 + nu * S3)[free]
    b = S1[free]
    c = (S2 + S4)[free] if use_s else np.zeros(n)
    # strictly feasible start: max s s.t. M x = rhs, DMIN + s <= x <= DMAX - s
    cost = np.zeros(n + 1)
    cost[-1] = -1.0
    A_ub = np.zeros((2 * n, n + 1))
    A_ub[:n, :n] = -np.eye(n)
    A_ub[:n, -1] = 1.0
    A_ub[n:, :n] = np.eye(n)
    A_ub[n:, -1] = 1.0
    b_ub = np.concatenate([np.full(n, -DMIN), np.full(n, DMAX)])
    A_eq = np.hstack([M, np.zeros((len(rhs), 1))]) if len(rhs) else None
    lp = optimize.linprog(cost, A_ub=A_ub, b_ub=b_ub, A_eq=A_eq,
                          b_eq=rhs if len(rhs) else None,
                          bounds=[(None, None)] * n + [(None, (DMAX - DMIN) / 2)],
                          method="highs")
    if lp.status != 0 or lp.x[-1] <= 1e-12:
        return out, False
    x = lp.x[:n].copy()
    Z = linalg.null_space(M) if len(rhs) else np.eye(n)
    if Z.shape[1] == 0:
        out[free] = x
        return out, True

    def fval(x):
        v = -a * x + b * _log1mexp(x)
        if use_s:
            v = v + c * _log1mexp(nu * x)
        return float(np.sum(v))

    def derivs(x):
        e = np.expm1(x)
        g = -a + b / e
        h = -b * (e + 1) / (e * e)
        if use_s:
            en = np.expm1(nu * x)
            g = g + c * nu / en
            h = h - c * nu * nu * (en + 1) / (en * en)
        return g, h

    def barrier(x, t):
        return t * fval(x) + float(np.sum(np.log(x - DMIN) + np.log(DMAX - x)))

    m = 2.0 * n
    tol = 1e-11 * (abs(fval(x)) + 1.0)
    t = 1.0
    for _ in range(60):
        for _ in range(100):
            g, h = derivs(x)
            gb = t * g + 1.0 / (x - DMIN) - 1.0 / (DMAX - x)
            hb = t * h - 1.0 / (x - DMIN) ** 2 - 1.0 / (DMAX - x) ** 2
            gy = Z.T @ gb
            Hy = (Z.T * -hb) @ Z
            dy = np.linalg.solve(Hy, gy)
            lam2 = float(gy @ dy)
            if lam2 / 2 <= 1e-12:
                break
            dx = Z @ dy
            with np.errstate(divide="ignore"):
                lim = np.where(dx > 0, (DMAX - x) / dx, np.where(dx < 0, (x - DMIN) / -dx, np.inf))
            alpha = min(1.0, 0.99 * float(np.min(lim)))
            f0 = barrier(x, t)
            while alpha > 1e-20 and barrier(x + alpha * dx, t) < f0 + 0.25 * alpha * lam2:
                alpha *= 0.5
            if alpha <= 1e-20:
                break
            x = x + alpha * dx
        if m / t <= tol:
            break
        t *= 10.0
    out[free] = np.clip(x, DMIN, DMAX)
    return out, True


# ----------------------------------------------------------------------------
# EM loops
# ----------------------------------------------------------------------------
# ----------------------------------------------------------------------------
# fastEM's own M-step: 100 steps of L-BFGS with a line search on
# M_step_loss_fn in (log d, logit nu, logit phi), FP32 (fast_em/laml.py:49-110).
# The reference runs optax (>= 0.2.4, < 1.0; not vendored): optax.lbfgs with
# scale_init_precond=True -- the two-loop recursion over the last 10 pairs,
# the initial inverse Hessian <s, y> / <y, y> of the newest pair -- and its
# default zoom line search (strong Wolfe, c1 = 1e-4, c2 = 0.9, first trial
# step 1, at most 20 evaluations), chained with
# scale_by_backtracking_linesearch(15): an Armijo test (slope 1e-4) on the
# step found, shrunk by 0.8 up to 15 times.  This restates those published
# methods (Nocedal & Wright, Numerical Optimization, algorithms 3.5, 3.6 and
# 7.4); optax's own iterates are not reproduced bit for bit (parity unpinned).
# ----------------------------------------------------------------------------
LBFGS_STEPS = 100          # M_STEP_DESCENT_STEPS, fast_em/laml.py:44
LBFGS_MEMORY = 10
WOLFE_C1, WOLFE_C2, ZOOM_EVALS = 1e-4, 0.9, 20
BACKTRACK_STEPS, BACKTRACK_FACTOR = 15, 0.8


def mstep_loss_grad(x, counts, leaf_resp_total, R, M, branch_mask, param_mask):
    """M_step_loss_fn (fast_em/laml.py:62-78) and its gradient in FP32 at
    x = (log d [N], logit nu, logit phi); the gradient is masked as
    laml.py:88-92 masks it."""
    f32 = np.float32
    x = np.asarray(x, dtype=f32)
    N = x.shape[0] - 2
    lo = f32(math.log(CALC_EPS))
    u = x[:N]
    d = np.exp(np.clip(u, lo, -lo))
    sd = (u > lo) & (u < -lo)
    with np.errstate(over="ignore"):
        sig = f32(1) / (f32(1) + np.exp(-x[N:]))
    mp = np.clip(sig, f32(CALC_EPS), f32(1 - CALC_EPS))
    sm = (sig > f32(CALC_EPS)) & (sig < f32(1 - CALC_EPS))
    nu, phi = mp[0], mp[1]
    e = np.asarray(counts, dtype=f32)
    ln2 = f32(math.log(2.0))

    def l1m(z):   # log(1 - e^-z), fast_em's log1mexp_pos
        with np.errstate(divide="ignore", invalid="ignore"):
            return np.where(z > ln2, np.log1p(-np.exp(-z)), np.log(-np.expm1(-z)))

    dn = d * nu
    c1 = -e[:, 0] * d * (f32(1) + nu)
    c2 = e[:, 1] * (l1m(d) - d * nu)
    c3 = e[:, 2] * l1m(dn)
    c4 = -e[:, 3] * d * nu
    c5 = e[:, 4] * l1m(dn)
    R32, M32, LR = f32(R), f32(M), f32(leaf_resp_total)
    c6 = R32 * np.log(f32(1) - phi) + (M32 - LR) * np.log(phi)
    loss = -(np.sum(c1 + c2 + c3 + c4 + c5, dtype=f32) + c6)
    with np.errstate(divide="ignore", over="ignore"):
        ie = f32(1) / np.expm1(d)
        ien = f32(1) / np.expm1(dn)
    cs = e[:, 2] + e[:, 4]
    dfd = -e[:, 0] * (f32(1) + nu) + e[:, 1] * (ie - nu) + cs * nu * ien - e[:, 3] * nu
    dfn = np.sum(-(e[:, 0] + e[:, 1] + e[:, 3]) * d + cs * d * ien, dtype=f32)
    dfp = -R32 / (f32(1) - phi) + (M32 - LR) / phi
    g = np.empty_like(x)
    g[:N] = np.where(sd, -dfd * d, f32(0)) * np.asarray(branch_mask, dtype=f32)
    gm = np.array([-dfn, -dfp], dtype=f32) * mp * (f32(1) - mp)
    g[N:] = np.where(sm, gm, f32(0)) * np.asarray(param_mask, dtype=f32)
    return f32(loss), g


def _cubic_step(lo, flo, dlo, hi, fhi, dhi):
    """Minimiser of the cubic through (lo, flo, dlo), (hi, fhi, dhi) (Nocedal
    & Wright eq. 3.59), kept inside the bracket by 10% of its width;
    bisection where the cubic has no usable minimiser."""
    w = abs(hi - lo)
    if np.isfinite(fhi) and np.isfinite(dhi) and w > 0:
        d1 = dlo + dhi - 3 * (flo - fhi) / (lo - hi)
        rad = d1 * d1 - dlo * dhi
        if rad >= 0:
            d2 = math.copysign(math.sqrt(rad), hi - lo)
            den = dhi - dlo + 2 * d2
            if den != 0:
                a = hi - (hi - lo) * (dhi + d2 - d1) / den
                if min(lo, hi) + 0.1 * w <= a <= max(lo, hi) - 0.1 * w:
                    return a
    return 0.5 * (lo + hi)


def _zoom_search(fg, x, f0, g0, p):
    """A step along p meeting the strong Wolfe conditions: first trial 1,
    doubled while the slope stays negative, then the zoom of the bracket;
    at most ZOOM_EVALS evaluations.  Returns (step, f, g); on exhaustion the
    best point with sufficient decrease seen, else the last trial."""
    d0 = float(np.dot(g0, p))
    st = {"n": 0, "best": None}

    def ev(a):
        st["n"] += 1
        f, g = fg(x + np.float32(a) * p)
        f = float(f)
        if np.isfinite(f) and f <= f0 + WOLFE_C1 * a * d0 and (
                st["best"] is None or f < st["best"][1]):
            st["best"] = (a, f, g)
        return f, g, float(np.dot(g, p))

    def zoom(lo, flo, dlo, hi, fhi, dhi):
        last = None
        while st["n"] < ZOOM_EVALS:
            a = _cubic_step(lo, flo, dlo, hi, fhi, dhi)
            f, g, da = ev(a)
            last = (a, f, g)
            if not np.isfinite(f) or f > f0 + WOLFE_C1 * a * d0 or f >= flo:
                hi, fhi, dhi = a, f, da
            else:
                if abs(da) <= -WOLFE_C2 * d0:
                    return a, f, g
                if da * (hi - lo) >= 0:
                    hi, fhi, dhi = lo, flo, dlo
                lo, flo, dlo = a, f, da
        return st["best"] if st["best"] is not None else last

    a_prev, f_prev, d_prev = 0.0, f0, d0
    a = 1.0
    while st["n"] < ZOOM_EVALS:
        f, g, da = ev(a)
        if not np.isfinite(f) or f > f0 + WOLFE_C1 * a * d0 or (a_prev > 0 and f >= f_prev):
            return zoom(a_prev, f_prev, d_prev, a, f, da)
        if abs(da) <= -WOLFE_C2 * d0:
            return a, f, g
        if da >= 0:
            return zoom(a, f, da, a_prev, f_prev, d_prev)
        a_prev, f_prev, d_prev = a, f, da
        a = 2.0 * a
    if st["best"] is not None:
        return st["best"]
    return a_prev, f_prev, fg(x + np.float32(a_prev) * p)[1]


def lbfgs_start(d, nu, phi):
    """The EM loop's parameter vector (fast_em/laml.py:126-139): log max(d,
    EPS) and the logits of nu and phi clamped to [EPS, 1 - EPS], FP32."""
    N = len(d)
    x = np.empty(N + 2, dtype=np.float32)
    x[:N] = np.log(np.maximum(np.asarray(d, dtype=np.float64), EPS))
    nu = min(max(nu, EPS), 1 - EPS)
    phi = min(max(phi, EPS), 1 - EPS)
    x[N] = math.log(nu / (1 - nu))
    x[N + 1] = math.log(phi / (1 - phi))
    return x


def lbfgs_params(x):
    """(d, nu, phi) of a parameter vector as the E-step reads them:
    exp(log d), sigmoid(logits), unclamped (laml.py:151-156)."""
    x = np.asarray(x, dtype=np.float64)
    N = len(x) - 2
    with np.errstate(over="ignore"):
        mp = 1.0 / (1.0 + np.exp(-x[N:]))
    return np.exp(x[:N]), float(mp[0]), float(mp[1])


def mstep_compat_lbfgs(counts, leaf_resp_total, R, M, x, branch_mask, fix_nu, fix_phi,
                       steps=LBFGS_STEPS):
    """fastEM's M-step as the reference runs it (fast_em/laml.py:84-110): 100
    L-BFGS steps with the zoom line search and the chained backtracking
    test, from the EM loop's parameter vector x (log d, logit nu, logit
    phi; the loop keeps it across iterations, laml.py:190).  Returns the new
    vector."""
    f32 = np.float32
    x = np.asarray(x, dtype=f32).copy()
    pm = np.array([0.0 if fix_nu else 1.0, 0.0 if fix_phi else 1.0], dtype=f32)
    bm = np.asarray(branch_mask, dtype=f32)

    def fg(z):
        return mstep_loss_grad(z, counts, leaf_resp_total, R, M, bm, pm)

    f, g = fg(x)
    S, Y, W = [], [], []
    for _ in range(steps):
        q = g.copy()
        al = []
        for s_, y_, w_ in zip(reversed(S), reversed(Y), reversed(W)):
            a = w_ * f32(np.dot(s_, q))
            q = q - a * y_
            al.append(a)
        gam = f32(1)
        if S:
            yy = f32(np.dot(Y[-1], Y[-1]))
            if yy > 0:
                gam = f32(np.dot(S[-1], Y[-1])) / yy
        z = gam * q
        for (s_, y_, w_), a in zip(zip(S, Y, W), reversed(al)):
            z = z + s_ * (a - w_ * f32(np.dot(y_, z)))
        p = -z
        if not float(np.dot(g, p)) < 0:   # not a descent direction: the gradient
            p = -g
            S, Y, W = [], [], []
        if not float(np.dot(g, p)) < 0:
            break                          # stationary under the masks
        a, fn, gn = _zoom_search(fg, x, float(f), g, p)
        u = np.float32(a) * p
        slope = float(np.dot(g, u))       # the chained backtracking test
        t = 1.0
        for _ in range(BACKTRACK_STEPS):
            if np.isfinite(fn) and fn <= float(f) + 1e-4 * t * slope:
                break
            t *= BACKTRACK_FACTOR
            fn, gn = fg(x + np.float32(t) * u)
            fn = float(fn)
        xn = x + np.float32(t) * u
        s_, y_ = xn - x, gn - g
        sy = f32(np.dot(s_, y_))
        S.append(s_)
        Y.append(y_)
        W.append(f32(0) if sy == 0 else f32(1) / sy)
        if len(S) > LBFGS_MEMORY:
            S.pop(0), Y.pop(0), W.pop(0)
        x, f, g = xn, f32(fn), gn
    return x


@dataclass
class EMResult:
    llh: float
    d: np.ndarray
    nu: float
    phi: float
    iterations: int
    trace: List[float] = field(default_factory=list)
    status: str = "optimal"


def em_compat(prob: Problem, d, nu, phi, branch_mask=None, fix_nu=False, fix_phi=False,
              max_iters=10_000, rounds=MSTEP_ROUNDS, stop=EM_STOP_COMPAT,
              mstep="stationary") -> EMResult:
    """optimize_parameters_expectation_maximization (fast_em/laml.py:112-194)
    with ``mstep`` "stationary" (the M-step objective solved to its
    stationary point) or "lbfgs" (the reference's 100 L-BFGS steps,
    ``mstep_compat_lbfgs``, the parameter vector kept across iterations):
    clamp nu, phi to [EPS, 1-EPS], floor d at EPS, loop E -> M -> logL until
    the relative change is below 1e-5; on convergence return the new logL
    with the parameters *before* the last M-step (the loop breaks before
    ``params = new_params``); a NaN keeps the previous logL."""
    N = len(prob.tree.parent)
    nu = min(max(nu, EPS), 1 - EPS)
    phi = min(max(phi, EPS), 1 - EPS)
    d = np.maximum(np.asarray(d, dtype=np.float64), EPS)
    mask = np.ones(N, dtype=bool) if branch_mask is None else np.asarray(branch_mask, bool)
    chars = prob.enc.chars
    M = float(np.sum(chars == MISSING))
    R = float(np.sum(chars != MISSING))
    x = lbfgs_start(d, nu, phi) if mstep == "lbfgs" else None
    if x is not None:
        d, nu, phi = lbfgs_params(x)
    prev, _ = log_likelihood(prob, d, nu, phi)
    trace = [prev]
    it = 0
    cur = prev
    while it < max_iters:
        it += 1
        es = e_step(prob, d, nu, phi)
        if x is not None:
            xn = mstep_compat_lbfgs(es.counts, float(es.leaf_resp.sum()), R, M, x, mask,
                                    fix_nu, fix_phi)
            dn, nun, phin = lbfgs_params(xn)
        else:
            dn, nun, phin = mstep_compat(es.counts, float(es.leaf_resp.sum()), R, M, d, nu,
                                         phi, mask, fix_nu, fix_phi, rounds=rounds)
        cur, _ = log_likelihood(prob, dn, nun, phin)
        trace.append(cur)
        if abs(cur - prev) / abs(prev) < stop:
            break
        if math.isnan(cur):
            cur = prev
            break
        d, nu, phi = dn, nun, phin
        if x is not None:
            x = xn
        prev = cur
    return EMResult(cur, d, nu, phi, it, trace)


def exact_leaf_stats(prob: Problem, es: EStep):
    """(sum over '?' leaf entries of P(silenced|D), number of '?' entries) and
    R = number of non-'?' leaf entries (EM_solver.py:318-324)."""
    n = prob.tree.num_leaves
    ch = prob.enc.chars
    miss = ch == MISSING
    p1 = np.exp(es.post1[:n])
    return (float(np.sum(p1[miss])), float(np.sum(miss))), float(np.sum(~miss))


def em_exact(prob: Problem, d, nu, phi, branch_mask=None, fix_nu=False, fix_phi=False,
             max_iters=1000, stop=None, ultra=False) -> EMResult:
    """EM_solver.EM_optimization (EM_solver.py:461-512): E-step, M-step,
    logL; stop when |(cur-pre)/pre| < conv_eps = 1e-8 (``stop``; negative:
    never) or after 1000 iterations.  ``ultra``: M-steps under the
    ultrametric equalities; a failed solve ends the EM with the
    log-likelihood before it and status "d_infeasible" (EM_solver.py:491-495)."""
    stop = CONV_EPS_EXACT if stop is None else stop
    N = len(prob.tree.parent)
    d = np.asarray(d, dtype=np.float64).copy()
    mask = np.ones(N, dtype=bool) if branch_mask is None else np.asarray(branch_mask, bool)
    K = prob.enc.chars.shape[1]
    ncells = prob.tree.num_leaves
    pre, _ = log_likelihood(prob, d, nu, phi)
    trace = [pre]
    it = 1
    cur = pre
    while it <= max_iters:
        es = e_step(prob, d, nu, phi)
        lstat, R = exact_leaf_stats(prob, es)
        out = mstep_exact(es.counts, lstat, R, d, nu, phi, mask, K, ncells,
                          opt_phi=not fix_phi, opt_nu=not fix_nu,
                          ultra_tree=prob.tree if ultra else None)
        if ultra and not out[3]:
            return EMResult(pre, d, nu, phi, it, trace, "d_infeasible")
        d, nu, phi = out[:3]
        cur, _ = log_likelihood(prob, d, nu, phi)
        trace.append(cur)
        if abs((cur - pre) / pre) < stop:
            break
        pre = cur
        it += 1
    return EMResult(cur, d, nu, phi, it, trace)


def em_exact_forest(probs: Sequence[Problem], ds, nu, phi, masks=None, fix_nu=False,
                    fix_phi=False, max_iters=1000, stop=None, ultra=False,
                    ncells=None) -> EMResult:
    """EM_solver.EM_optimization with several trees (EM_solver.py:461-512):
    every tree's E-step, one M-step over all of them (phi from all leaves,
    every branch, one nu; EM_solver.py:307-459), the stopping rule on the
    summed log-likelihood; with ``ultra`` the branch lengths under every
    tree's equalities and the root rows that tie the trees together
    (ultrametric_constraints_forest).  ``ncells``: the character matrix's
    cells (the phi zero threshold, 1 / (sites x cells)); default the first
    tree's leaves.  The result's ``d`` is the list of the trees' lengths."""
    stop = CONV_EPS_EXACT if stop is None else stop
    k = len(probs)
    ds = [np.asarray(x, dtype=np.float64).copy() for x in ds]
    masks = [np.ones(len(p.tree.parent), bool) if masks is None else np.asarray(masks[i], bool)
             for i, p in enumerate(probs)]
    K = probs[0].enc.chars.shape[1]
    ncells = probs[0].tree.num_leaves if ncells is None else ncells
    sizes = [len(p.tree.parent) for p in probs]
    cuts = np.cumsum([0] + sizes)

    def llh_all(ds_, nu_, phi_):
        return sum(log_likelihood(p, d_, nu_, phi_)[0] for p, d_ in zip(probs, ds_))

    pre = llh_all(ds, nu, phi)
    trace = [pre]
    it, cur = 1, pre
    while it <= max_iters:
        counts, ls, lc, R = [], 0.0, 0.0, 0.0
        for p, d_ in zip(probs, ds):
            es = e_step(p, d_, nu, phi)
            (a, c), r = exact_leaf_stats(p, es)
            counts.append(es.counts)
            ls, lc, R = ls + a, lc + c, R + r
        cons = (ultrametric_constraints_forest([p.tree for p in probs], masks, ds)
                if ultra else None)
        out = mstep_exact(np.concatenate(counts), (ls, lc), R, np.concatenate(ds), nu, phi,
                          np.concatenate(masks), K, ncells, opt_phi=not fix_phi,
                          opt_nu=not fix_nu, ultra_constraints=cons)
        if ultra and not out[3]:
            return EMResult(pre, ds, nu, phi, it, trace, "d_infeasible")
        dcat, nu, phi = out[:3]
        ds = [dcat[cuts[i]:cuts[i + 1]].copy() for i in range(k)]
        cur = llh_all(ds, nu, phi)
        trace.append(cur)
        if abs((cur - pre) / pre) < stop:
            break
        pre = cur
        it += 1
    return EMResult(cur, ds, nu, phi, it, trace)


def exact_initials(tree: ParsedTree, N_postorder_lengths, randseed, fixed_phi=None,
                   fixed_nu=None):
    """ML_solver.ini_all under ``seed(randseed)`` (ML_solver.py:195-213):
    uniform draws for every edge (postorder), replaced by max(2 dmin, length)
    where a length exists; then nu and phi = random()*0.99 unless fixed."""
    rs = _random.Random(randseed)
    ne = len(N_postorder_lengths)
    x = [rs.random() * (DMAX / 2 - 2 * DMIN) + 2 * DMIN for _ in range(ne)]
    for i, L in enumerate(N_postorder_lengths):
        if L is not None:
            x[i] = max(2 * DMIN, L)
    nu = rs.random() * 0.99 if fixed_nu is None else fixed_nu
    phi = rs.random() * 0.99 if fixed_phi is None else fixed_phi
    return x, nu, phi


def treeswift_postorder_ids(tree: ParsedTree) -> List[int]:
    """parse_tree ids in treeswift postorder of the same tree (children in
    newick order, i.e. the reverse of the networkx successor order): the order
    of EM_solver's parameter vector (ML_solver.py:195-203, 231-236)."""
    out, st = [], [(tree.root, False)]
    while st:
        u, done = st.pop()
        if done:
            out.append(u)
            continue
        st.append((u, True))
        for c in tree.children[u]:
            st.append((c, False))
    return out


# ----------------------------------------------------------------------------
# annotations (runner.py:367-435)
# ----------------------------------------------------------------------------
def az_labels(prob: Problem):
    """ML_solver.az_partition (ML_solver.py:125-154) on the recoded matrix:
    per (node, site) 'z', '?' or the recoded state."""
    tr, ch = prob.tree, prob.enc.chars
    N, n, K = len(tr.parent), tr.num_leaves, ch.shape[1]
    lab = [[None] * K for _ in range(N)]
    for u in _postorder_ids(tr):
        if u < n:
            for c in range(K):
                x = int(ch[u, c])
                lab[u][c] = "z" if x == 0 else ("?" if x < 0 else x)
        else:
            for c in range(K):
                S = set(lab[v][c] for v in tr.children[u])
                Rr = S - {"z", "?"}
                if "z" in S or len(Rr) > 1:
                    lab[u][c] = "z"
                elif len(Rr) == 1:
                    lab[u][c] = next(iter(Rr))
                else:
                    lab[u][c] = "?"
    return lab


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


def annotation_strings(prob: Problem, post0, post1, Q):
    """Per node (parse_tree id order) the comma-joined posterior strings of
    runner.py:414-430; '?' clades inherit the parent's alpha when it is not
    'z'; the alpha is printed in the original state space."""
    tr = prob.tree
    lab = az_labels(prob)
    K = prob.enc.chars.shape[1]
    for u in _preorder_ids(tr):
        p = tr.parent[u]
        if p >= 0:
            for c in range(K):
                if lab[u][c] == "?" and lab[p][c] != "z":
                    lab[u][c] = lab[p][c]
    out = {}
    for u in range(len(tr.parent)):
        parts = []
        for c in range(K):
            p0 = round(math.exp(post0[u, c]), 2)
            pm = round(math.exp(post1[u, c]), 2)
            pa = round(1 - p0 - pm, 2)
            a = lab[u][c]
            if isinstance(a, (int, np.integer)):
                a = str(prob.enc.state_maps[c][int(a) - 1])
            parts.append(format_posterior(p0, pm, pa, str(a), Q[c]))
        out[tr.labels[u]] = ",".join(parts)
    return out
