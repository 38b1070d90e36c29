"""Drop-in mirror of laml_libs/fastEM_solver.py on the GB300 engine.

Same constructor and methods as the reference solver (Virtual_solver /
ML_solver / EM_solver / fastEM_solver, laml_libs/*.py):

* ``fastEM_solver(treeList, data, prior, params)`` -- ``treeList`` newick
  strings; ``data = {'charMtrx': {cell: [int|'?']}, 'ordered_leaf_labels':
  [[...]], ...}``; ``prior = {'Q': [{state: prob}], ...}``.
* ``score_tree(strategy) -> (score, status)``: the fastEM path
  (fastEM_solver.py:283-353): each tree runs fastEM's EM from nu = phi = 0.5
  (or the fixed values given), branch lengths written back; with
  ``'final_optimization'`` in the strategy the exact EM (EM_solver) runs
  instead (fastEM_solver.py:295-297).
* ``negative_llh()``: the exact-model log-likelihood (ML_solver.py:252-254,
  EM_solver.py:135-141).
* ``optimize(initials, fixed_phi, fixed_nu, fixed_brlen, verbose, max_trials,
  random_seeds, ultra_constr)``: the exact EM with EM_solver's initial points
  (ML_solver.py:256-336, EM_solver.py:514-527).
* ``get_params()``, ``get_tree_newick()``, ``params.nu`` / ``params.phi``.

Every likelihood, E-step and M-step runs on the GPU; there is no CPU path.
Only binary trees are supported (a polytomy raises ValueError).  With
``ultra_constr=True`` every M-step solves the branch lengths under
EM_solver's ultrametric equalities (EM_solver.py:53-89, 358-361) on the
device.  Several trees share one nu and one phi and run one EM on their
summed log-likelihood, as EM_solver's M-step over all of its trees does
(EM_solver.py:307-459), with their roots at one height under
``ultra_constr`` (EM_solver.py:81-84): the trees are joined under
zero-length fixed branches (laml_gb300/forest.py).  Constraints without a
solution end the EM with status "d_infeasible", as
EM_solver.EM_optimization does (EM_solver.py:491-495).
"""
from __future__ import annotations

import random as _random
from typing import List, Optional

import numpy as np

from .encoding import EncodedTree, char_matrix, encode_dataset, encode_newick
from ._native import TREE_INFEASIBLE
from .forest import join_forest
from .engine import MSTEP_ROUNDS, DeviceBatch
from .fast_em.phylogeny import Phylogeny, build_phylogeny, tree_to_networkx

EPS_PARAM = 1e-10          # laml_libs/core_constants.py:4 (eps)
DMIN, DMAX = 0.005, 10.0   # laml_libs/core_constants.py:7-8


class Params:
    def __init__(self, nu, phi):
        self.nu = nu
        self.phi = phi


def write_newick(et: EncodedTree, d: Optional[np.ndarray] = None) -> str:
    """Newick of an encoded tree (children in their newick order, every node
    labelled, lengths from ``d`` or the tree)."""
    d = et.branch_length if d is None else d
    root = et.root
    out = []
    st = [(root, 0)]
    while st:
        u, k = st.pop()
        if et.child0[u] < 0:
            out.append(f"{et.labels[u]}:{float(d[u])!r}")
            continue
        ch = (int(et.child1[u]), int(et.child0[u]))   # newick order
        if k == 0:
            out.append("(")
        if k < 2:
            if k > 0:
                out.append(",")
            st.append((u, k + 1))
            st.append((ch[k], 0))
        else:
            out.append(f"){et.labels[u]}:{float(d[u])!r}")
    return "".join(out) + ";"


def parse_tree(tree, has_branch_mask=False, ordered_leaf_labels=None, fixed=None,
               rng=None) -> dict:
    """fastEM_solver.parse_tree (fastEM_solver.py:46-146) for a newick string
    (or an object with ``.newick()``): the networkx tree, branch lengths
    (U(0.01, 0.5) where missing, leaves first), the branch mask (True = free;
    ``fixed`` is the set of labels marked fixed) and the relabeling vector."""
    nw = tree if isinstance(tree, str) else tree.newick()
    et = encode_newick(nw, ordered_leaf_labels)
    rng = rng if rng is not None else _random
    bl = et.branch_length.copy()
    for i in range(et.num_nodes):
        if not et.has_length[i]:
            bl[i] = rng.uniform(0.01, 0.5)
    if has_branch_mask:
        fixed = fixed or set()
        mask = np.array([lab not in fixed for lab in et.labels])
    else:
        mask = np.ones(et.num_nodes, bool)
    return {"nxtree": tree_to_networkx(et), "num_leaves": et.num_leaves, "branch_lengths": bl,
            "branch_mask": mask, "relabeling_vector": list(et.labels), "encoded": et}


def parse_data(parser_tree_out, data, prior) -> Phylogeny:
    """fastEM_solver.parse_data (fastEM_solver.py:17-44)."""
    order = parser_tree_out["relabeling_vector"][:parser_tree_out["num_leaves"]]
    rows = {c: data["charMtrx"][c] for c in order}
    pri = {}
    for c, q in enumerate(prior["Q"]):
        for s, p in q.items():
            pri[(c, int(s))] = float(p)
    return build_phylogeny(parser_tree_out["nxtree"], parser_tree_out["num_leaves"], rows, pri)


def _lca(et: EncodedTree, a: int, b: int) -> int:
    seen = set()
    x = a
    while x >= 0:
        seen.add(x)
        x = int(et.parent[x])
    x = b
    while x not in seen:
        x = int(et.parent[x])
    return x


class fastEM_solver:
    """The reference solver's interface, every computation on the GPU.

    ``mstep`` (class attribute) picks the fastEM M-step: "stationary" solves
    the M_step_loss_fn objective to its stationary point; "lbfgs" runs the
    reference's own 100 FP32 L-BFGS steps (fast_em/laml.py:84-110,
    LAML_MSTEP_LBFGS), which may stop short of that point."""

    mstep = "stationary"

    def __init__(self, treeList, data, prior, params={'nu': 0, 'phi': 0, 'sigma': 0},
                 group_sites: int = 8, device="cuda"):
        self.solver_name = "fastEM_solver"
        self.data, self.prior = data, prior
        self.charMtrx = data["charMtrx"]
        self.Q = prior["Q"]
        self.treeList = [t if isinstance(t, str) else t.newick() for t in treeList]
        # fastEM_solver passes nu = phi = 0 to its parents (fastEM_solver.py:152)
        self.params = Params(0, 0)
        self.numsites = len(next(iter(self.charMtrx.values())))
        self.G, self.device = group_sites, device
        order = data.get("ordered_leaf_labels")
        self.ordered_leaf_labels = []
        self.trees: List[EncodedTree] = []
        for i, nw in enumerate(self.treeList):
            lo = order[i] if order is not None else None
            et = encode_newick(nw, lo)
            if lo is None:
                lo = et.labels[:et.num_leaves]
            self.ordered_leaf_labels.append(list(lo))
            self.trees.append(et)
        self._d = [t.branch_length.copy() for t in self.trees]
        for t, d in zip(self.trees, self._d):
            for i in np.flatnonzero(~t.has_length):
                d[i] = _random.uniform(0.01, 0.5)
        self._ds_cache = {}

    # -- helpers --------------------------------------------------------
    def _dataset(self, tidx, compat):
        key = (tidx, compat)
        if key not in self._ds_cache:
            lo = self.ordered_leaf_labels[tidx]
            mat = char_matrix([self.charMtrx[c] for c in lo], exact=not compat)
            self._ds_cache[key] = encode_dataset(mat, self.Q, compat=compat, group_sites=self.G)
        return self._ds_cache[key]

    def _fixed_mask(self, tidx, fixed_brlen):
        """Branches fixed by ``fixed_brlen[tidx]``: {(leafA, leafB): length}
        fixes the edge above LCA(leafA, leafB) (ML_solver.py:296-305)."""
        et = self.trees[tidx]
        mask = np.ones(et.num_nodes, bool)
        d = self._d[tidx]
        if fixed_brlen is None:
            return mask
        lab = {l: i for i, l in enumerate(et.labels)}
        for (a, b), L in fixed_brlen[tidx].items():
            u = _lca(et, lab[a], lab[b])
            mask[u] = False
            d[u] = L
        return mask

    # -- Virtual_solver / ML_solver surface -------------------------------
    def get_tree_newick(self):
        return [write_newick(t, d) for t, d in zip(self.trees, self._d)]

    def get_params(self):
        return {'phi': self.params.phi, 'nu': self.params.nu}

    def negative_llh(self):
        """EM_solver.lineage_llh at the current parameters (exact model)."""
        total = 0.0
        for i, t in enumerate(self.trees):
            b = DeviceBatch([self._dataset(i, False)], [t], [0], [self._d[i]],
                            [self.params.nu], [self.params.phi], compat=False,
                            device=self.device)
            total += float(b.log_likelihood()[0])
        return -total

    def score_tree(self, strategy={'ultra_constr': False, 'fixed_phi': None, 'fixed_nu': None,
                                   'fixed_brlen': None, 'nodes_to_recompute': None}):
        if 'final_optimization' in strategy:
            return self.score_tree_oldEM(strategy)
        fixed_phi, fixed_nu = strategy.get('fixed_phi'), strategy.get('fixed_nu')
        has_mask = strategy.get('fixed_brlen') is not None
        score = None
        for i, t in enumerate(self.trees):
            # fastEM_solver.py:310-316: every node is marked fixed and the
            # recompute test compares a label with node objects, so with
            # fixed_brlen given no branch length is freed
            mask = np.zeros(t.num_nodes, bool) if has_mask else np.ones(t.num_nodes, bool)
            nu = fixed_nu if fixed_nu else 0.5
            phi = fixed_phi if fixed_phi else 0.5
            b = DeviceBatch([self._dataset(i, True)], [t], [0],
                            [np.maximum(self._d[i], 1e-6)],
                            [min(max(nu, 1e-6), 1 - 1e-6)], [min(max(phi, 1e-6), 1 - 1e-6)],
                            compat=True, mask=[mask], device=self.device)
            b.lbfgs = self.mstep == "lbfgs"
            r = b.run_em(rounds=MSTEP_ROUNDS)[0]
            self.params.nu, self.params.phi = r.nu, r.phi
            self._d[i] = r.branch_lengths
            self.last_em_iterations = r.iterations
            score = r.llh
        return score, "optimal"

    def score_tree_oldEM(self, strategy):
        nllh, status = self.optimize(initials=1, verbose=-1,
                                     ultra_constr=strategy.get('ultra_constr', False),
                                     fixed_phi=strategy.get('fixed_phi'),
                                     fixed_nu=strategy.get('fixed_nu'),
                                     fixed_brlen=strategy.get('fixed_brlen'))
        return (None if nllh is None else -nllh), status

    def optimize(self, initials=20, fixed_phi=None, fixed_nu=None, fixed_brlen=None, verbose=1,
                 max_trials=100, random_seeds=None, ultra_constr=False):
        """EM_solver.optimize_one from ``initials`` starting points (the best
        nllh wins), seeds as ML_solver.optimize (ML_solver.py:263-282)."""
        if random_seeds is None:
            rseeds = [int(_random.random() * 10000) for _ in range(initials)]
        elif isinstance(random_seeds, int):
            _random.seed(a=random_seeds)
            rseeds = [int(_random.random() * 10000) for _ in range(initials)]
        else:
            rseeds = list(random_seeds)[:initials]
        best = None
        for rep in range(initials):
            res = self._optimize_one(rseeds[rep], fixed_phi, fixed_nu, fixed_brlen,
                                     ultra_constr)
            if best is None or res[0] < best[0]:
                best = res
        nllh, nu, phi, ds, status = best
        self.params = Params(nu, phi)
        self._d = ds
        return nllh, status

    def _optimize_one(self, randseed, fixed_phi, fixed_nu, fixed_brlen, ultra_constr=False):
        rs = _random.Random(randseed)
        ds, masks = [], []
        for i, t in enumerate(self.trees):
            masks.append(self._fixed_mask(i, fixed_brlen))
        # ML_solver.ini_all: one draw per edge (treeswift postorder), then nu, phi
        post = []
        for t in self.trees:
            post.append(_ts_postorder(t))
        ne = sum(len(p) for p in post)
        x = [rs.random() * (DMAX / 2 - 2 * DMIN) + 2 * DMIN for _ in range(ne)]
        nu = rs.random() * 0.99 if fixed_nu is None else fixed_nu
        phi = rs.random() * 0.99 if fixed_phi is None else fixed_phi
        k = 0
        for i, t in enumerate(self.trees):
            d = np.empty(t.num_nodes)
            for u in post[i]:
                has = t.has_length[u] or not masks[i][u]
                d[u] = max(2 * DMIN, self._d[i][u]) if has else x[k]
                k += 1
            ds.append(d)
        if len(self.trees) > 1:
            return self._optimize_forest(ds, masks, nu, phi, fixed_phi, fixed_nu, ultra_constr)
        total, out_d, status = 0.0, [], "optimal"
        for i, t in enumerate(self.trees):
            b = DeviceBatch([self._dataset(i, False)], [t], [0], [ds[i]], [nu], [phi],
                            compat=False, mask=[masks[i]], fix_nu=fixed_nu is not None,
                            fix_phi=fixed_phi is not None, device=self.device,
                            ultrametric=ultra_constr)
            r = b.run_em(max_iters=1000)[0]
            if r.status == TREE_INFEASIBLE:
                status = "d_infeasible"
            total += r.llh
            out_d.append(r.branch_lengths)
            nu, phi = r.nu, r.phi
        return -total, nu, phi, out_d, status


    def _optimize_forest(self, ds, masks, nu, phi, fixed_phi, fixed_nu, ultra_constr):
        """EM_solver's EM over all of its trees at once (one nu, one phi, the
        summed log-likelihood; with ultra_constr the trees' roots at one
        height, EM_solver.py:81-84): the trees joined under zero-length
        fixed branches (laml_gb300/forest.py), one device EM."""
        joined, maps, joins = join_forest(self.trees)
        rows = [self.charMtrx[c] for i in range(len(self.trees))
                for c in self.ordered_leaf_labels[i]]
        dset = encode_dataset(char_matrix(rows, exact=True), self.Q, compat=False,
                              group_sites=self.G)
        dj = np.zeros(joined.num_nodes)
        mj = np.zeros(joined.num_nodes, bool)
        for m, d, msk in zip(maps, ds, masks):
            dj[m] = d
            mj[m] = msk
        b = DeviceBatch([dset], [joined], [0], [dj], [nu], [phi], compat=False, mask=[mj],
                        fix_nu=fixed_nu is not None, fix_phi=fixed_phi is not None,
                        device=self.device, ultrametric=ultra_constr)
        r = b.run_em(max_iters=1000)[0]
        status = "d_infeasible" if r.status == TREE_INFEASIBLE else "optimal"
        return -r.llh, r.nu, r.phi, [r.branch_lengths[m].copy() for m in maps], status


def _ts_postorder(t: EncodedTree):
    """Node ids in treeswift postorder (children in newick order)."""
    out, st = [], [(t.root, False)]
    while st:
        u, done = st.pop()
        if done:
            out.append(u)
            continue
        st.append((u, True))
        if t.child0[u] >= 0:
            st.append((int(t.child0[u]), False))
            st.append((int(t.child1[u]), False))
    return out


class EM_solver(fastEM_solver):
    """Drop-in for laml_libs/EM_solver.py's solver class (``--solver EM``):
    ``score_tree(strategy)`` is ML_solver.score_tree (ML_solver.py:114-123),
    one exact EM from one initial point with the strategy's
    ``ultra_constr``, ``fixed_phi``, ``fixed_nu`` and ``fixed_brlen``; the
    rest of the interface is fastEM_solver's.  Binary trees only: the
    reference resolves polytomies into eps-length fixed branches
    (EM_solver.py:26-43); here a polytomy raises ValueError."""

    def __init__(self, treeList, data, prior, params={'nu': 0, 'phi': 0, 'sigma': 0},
                 group_sites: int = 8, device="cuda"):
        super().__init__(treeList, data, prior, params, group_sites=group_sites, device=device)
        self.solver_name = "EM_solver"

    def score_tree(self, strategy={'ultra_constr': False, 'fixed_phi': None, 'fixed_nu': None,
                                   'fixed_brlen': None}):
        return self.score_tree_oldEM(strategy)


class CandidateScore:
    """One candidate of score_candidate_batch: its fastEM score (the last
    tree's log-likelihood, as score_tree returns), parameters and -- built
    on first use -- its newick strings with the optimised branch lengths."""

    def __init__(self, score, params, topos, lengths, leaf_order):
        self.score = score
        self.params = params
        self._topos, self._lengths, self._leaf_order = topos, lengths, leaf_order
        self._newicks = None

    @property
    def newicks(self):
        if self._newicks is None:
            topos = self._topos() if callable(self._topos) else self._topos
            self._newicks = [write_newick(encode_newick(nw, self._leaf_order), d)
                             for nw, d in zip(topos, self._lengths)]
        return self._newicks


def score_candidate_batch(candidates, strategies, data, prior, params, group_sites=8,
                          device="cuda", trees=None):
    """fastEM_solver(treeList, data, prior, params).score_tree(strategy) for
    many candidates at once (each a treeList over the same leaves), as one
    batched EM on the device.  Per tree: missing lengths drawn U(0.01, 0.5) in
    node order (fastEM_solver.py:95-126, candidates in order), nu, phi start
    at the strategy's fixed values or 0.5 (320-321) and are optimised
    (323-324), every branch fixed when ``fixed_brlen`` is given (310-316).
    ``trees``: the candidates already encoded (one tree each, numbered in
    data['ordered_leaf_labels'] order, e.g. by laml_nni_candidates); each
    candidate is then a callable giving its newick list when it is needed."""
    from .encoding import encode_newick_batch
    lo = data.get("ordered_leaf_labels")
    leaf_order = list(lo[0]) if lo else None
    if trees is not None:
        if leaf_order is None:
            raise ValueError("encoded candidates need data['ordered_leaf_labels']")
        owner = list(range(len(trees)))
    else:
        flat, owner = [], []
        for ci, topos in enumerate(candidates):
            for nw in topos:
                flat.append(nw)
                owner.append(ci)
        if leaf_order is None:
            first = encode_newick(flat[0])
            leaf_order = first.labels[:first.num_leaves]
        trees = encode_newick_batch(flat, leaf_order)
    mat = char_matrix([data["charMtrx"][c] for c in leaf_order])
    ds = encode_dataset(mat, prior["Q"], compat=True, group_sites=group_sites)
    d, masks, nus, phis = [], [], [], []
    for t, ci in zip(trees, owner):
        st = strategies[ci]
        x = t.branch_length.copy()
        for i in np.flatnonzero(~t.has_length):
            x[i] = _random.uniform(0.01, 0.5)
        d.append(np.maximum(x, 1e-6))
        fixed = st.get('fixed_brlen') is not None
        masks.append(np.zeros(t.num_nodes, bool) if fixed else np.ones(t.num_nodes, bool))
        nu = st.get('fixed_nu') or 0.5
        phi = st.get('fixed_phi') or 0.5
        nus.append(min(max(nu, 1e-6), 1 - 1e-6))
        phis.append(min(max(phi, 1e-6), 1 - 1e-6))
    b = DeviceBatch([ds], trees, [0] * len(trees), d, nus, phis, compat=True, mask=masks,
                    device=device)
    b.lbfgs = fastEM_solver.mstep == "lbfgs"
    res = b.run_em(rounds=MSTEP_ROUNDS)
    out = []
    k = 0
    for ci, topos in enumerate(candidates):
        ntree = 1 if callable(topos) else len(topos)
        rs = res[k:k + ntree]
        k += ntree
        out.append(CandidateScore(rs[-1].llh, {'phi': rs[-1].phi, 'nu': rs[-1].nu}, topos,
                                  [r.branch_lengths for r in rs], leaf_order))
    return out
