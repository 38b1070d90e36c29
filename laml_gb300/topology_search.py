"""NNI topology search over the GPU solver.

``Topology_search`` keeps the interface and the search of
laml_libs/Topology_search.py (simulated-annealing acceptance, random branch
order, two NNI moves per internal edge, polytomy marking, local branch-length
strategy, checkpoints); it scores one candidate at a time through the solver
class it is given, as the reference does.

``Topology_search_batched`` is the GPU form of
laml_libs/Topology_search_parallel.py: it lists every NNI move of the current
trees in the same shuffled order, scores ``batch_size`` candidates at a time
in ONE batched EM on the device (all candidates share the encoded character
matrix; each keeps its own branch lengths, masks and parameters), and accepts
the first candidate of the batch that passes the acceptance rule -- the
parallel search's rule, with one device batch in place of a process pool.

Only the fastEM path (``fastEM_solver``) is batched; candidate scores follow
fastEM_solver.score_tree (fastEM_solver.py:283-353), including its handling
of ``fixed_brlen`` (every branch stays fixed when it is given).
"""
from __future__ import annotations

import random as _random
from copy import deepcopy
from math import exp
from typing import List

import numpy as np

from .tree import Node, Tree, find_lcas, read_tree_newick

DEFAULT_STRATEGY = {'resolve_search_only': False, 'only_marked': False, 'ultra_constr': False,
                    'fixed_phi': None, 'fixed_nu': None, 'local_brlen_opt': True,
                    'nodes_to_recompute': None}   # laml_libs/core_constants.py:10
CHKPT_FREQ = 10                                   # laml_libs/core_constants.py:9


def encoded_ids(tree: Tree, leaf_index) -> dict:
    """id(node) -> the node's id in laml_newick_encode's numbering of
    tree.newick(): leaves by ``leaf_index`` (label -> position), internal
    nodes in treeswift preorder (the traversal Tree.traverse_preorder
    makes).  None when the root is unifurcating (the encoder drops it)."""
    if len(tree.root.child_nodes()) == 1:
        return None
    out, nxt = {}, len(leaf_index)
    for node in tree.traverse_preorder():
        if node.is_leaf():
            out[id(node)] = leaf_index[node.label]
        else:
            out[id(node)] = nxt
            nxt += 1
    return out


class Topology_search:
    def __init__(self, treeTopoList, solver, data={}, prior={}, params={}, T_cooldown=20,
                 alpha_cooldown=0.9):
        self.treeTopoList = list(treeTopoList)
        self.solver = solver
        self.params = params
        self.data = data
        self.prior = prior
        self.__renew_treeList_obj__()
        self.has_polytomy = any(len(v.children) > 2 for t in self.treeList_obj
                                for v in t.traverse_preorder())
        self.treeTopoList = [t.newick() for t in self.treeList_obj]
        self.T_cooldown = T_cooldown
        self.alpha_cooldown = alpha_cooldown
        self.b = 1 / (1 - 1 / self.alpha_cooldown ** self.T_cooldown)
        self.a = -self.b / self.alpha_cooldown ** self.T_cooldown

    def __renew_treeList_obj__(self):
        self.treeList_obj = []
        for topo in self.treeTopoList:
            t = read_tree_newick(topo)
            t.suppress_unifurcations()
            self.treeList_obj.append(t)

    def get_solver(self):
        return self.solver(self.treeTopoList, self.data, self.prior, self.params)

    def update_from_solver(self, mySolver):
        self.treeTopoList = mySolver.get_tree_newick()
        self.params = mySolver.get_params()
        self.__renew_treeList_obj__()

    def __mark_polytomies__(self, eps_len=1e-3):
        self.has_polytomy = False
        for t in self.treeList_obj:
            for v in t.traverse_preorder():
                v.mark = False
                if len(v.children) > 2:
                    self.has_polytomy = True
            before = set(id(v) for v in t.traverse_preorder())
            t.resolve_polytomies()
            for v in t.traverse_preorder():
                if id(v) not in before:     # a node the resolution created
                    v.mark = True
                    v.edge_length = eps_len
        self.treeTopoList = [t.newick() for t in self.treeList_obj]

    def __accept_proposal__(self, curr_score, new_score, t):
        """Topology_search.py:78-90: better scores always; worse ones with
        probability exp((new - curr - 1e-12) / T), T = a alpha^t + b."""
        if new_score > curr_score:
            return True
        T = max(1e-12, self.a * self.alpha_cooldown ** t + self.b)
        p = min(exp((new_score - curr_score - 1e-12) / T), 1)
        return _random.random() < p

    def search(self, resolve_polytomies=True, maxiter=100, verbose=False, nreps=1,
               strategy=DEFAULT_STRATEGY, checkpoint_file=None):
        original_topos = self.treeTopoList
        original_params = self.params
        best_trees, best_score, best_params = None, -float("inf"), None
        for i in range(nreps):
            self.treeTopoList = original_topos
            self.params = original_params
            self.__renew_treeList_obj__()
            if resolve_polytomies:
                self.__mark_polytomies__()
            if strategy['resolve_search_only']:
                if self.has_polytomy:
                    trees, score, params = self.__search_one__(
                        strategy, maxiter=maxiter, verbose=verbose, only_marked=True,
                        checkpoint_file=checkpoint_file)
                else:
                    s = self.get_solver()
                    st = deepcopy(strategy)
                    st['fixed_brlen'] = None
                    st['nodes_to_recompute'] = None
                    score, status = s.score_tree(strategy=st)
                    self.update_from_solver(s)
                    trees, params = self.treeTopoList, self.params
            else:
                trees, score, params = self.__search_one__(
                    strategy, maxiter=maxiter, verbose=verbose, only_marked=False,
                    checkpoint_file=checkpoint_file)
            # final optimisation of the numerical parameters (Topology_search.py:146-158)
            self.treeTopoList = trees
            self.params = params
            self.__renew_treeList_obj__()
            s = self.get_solver()
            st = deepcopy(strategy)
            st['fixed_brlen'] = None
            st['final_optimization'] = True
            st['nodes_to_recompute'] = None
            score, status = s.score_tree(strategy=st)
            self.update_from_solver(s)
            trees, params = self.treeTopoList, self.params
            if verbose:
                print("Optimal score for this search: " + str(score), flush=True)
            if score > best_score:
                best_score, best_trees, best_params = score, trees, params
        self.treeTopoList = best_trees
        self.params = best_params
        return best_trees, best_score, best_params

    def __search_one__(self, strategy, maxiter=100, verbose=False, only_marked=False,
                       checkpoint_file=None):
        s = self.get_solver()
        st = deepcopy(strategy)
        st['fixed_brlen'] = None
        st['nodes_to_recompute'] = None
        curr_score, status = s.score_tree(strategy=st)
        if verbose:
            print("Initial score: " + str(curr_score), flush=True)
        self.update_from_solver(s)
        best_score, best_trees, best_params = curr_score, self.treeTopoList, self.params
        for nni_iter in range(maxiter):
            new_score, n_attempts, success = self.single_nni(curr_score, nni_iter, strategy,
                                                             only_marked=only_marked)
            if verbose:
                print(f"NNI Iter: {nni_iter}; trees checked: {n_attempts}", flush=True)
            if not success:
                break
            curr_score = new_score
            if curr_score > best_score:
                best_score, best_trees, best_params = curr_score, self.treeTopoList, self.params
            if nni_iter % CHKPT_FREQ == 0 and checkpoint_file is not None:
                with open(checkpoint_file, "a") as f:
                    f.write(f"NNI Iteration: {nni_iter}\n")
                    f.write(f"Current newick tree: {best_trees}\n")
                    f.write(f"Current negative-llh: {best_score}\n")
                    f.write(f"Current dropout rate: {best_params['phi']}\n")
                    f.write(f"Current silencing rate: {best_params['nu']}\n")
        return best_trees, best_score, best_params

    # -- moves -------------------------------------------------------------
    def _branches(self, only_marked):
        br = [v for t in self.treeList_obj for v in t.traverse_preorder()
              if not (v.is_leaf() or v.is_root()) and (not only_marked or v.mark)]
        _random.shuffle(br)
        return br

    def _local_strategy(self, u, v, strategy):
        """fixed_brlen / nodes_to_recompute of Topology_search.apply_nni
        (lines 256-289): every branch other than u's children, v's children
        and v is fixed at its current length, keyed by leaf anchors."""
        st = deepcopy(strategy)
        st['fixed_brlen'] = None
        st['nodes_to_recompute'] = None
        if not strategy['local_brlen_opt']:
            return st
        st['fixed_nu'] = self.params['nu']
        st['fixed_phi'] = self.params['phi']
        free = {id(x) for x in u.child_nodes() + v.child_nodes() + [v]}
        anchors = [[] for _ in self.treeList_obj]
        recompute = [[] for _ in self.treeList_obj]
        for t, tree in enumerate(self.treeList_obj):
            for node in tree.traverse_postorder():
                if node.is_leaf():
                    node.anchors = (node.label, node.label)
                else:
                    c = node.child_nodes()
                    node.anchors = (c[0].anchors[0], c[-1].anchors[0])
                (recompute if id(node) in free else anchors)[t].append(node.anchors)
        fixed_brlen = [{} for _ in self.treeList_obj]
        for t, topo in enumerate(self.treeTopoList):
            lcas = find_lcas(read_tree_newick(topo), anchors[t])
            for a, node in zip(anchors[t], lcas):
                fixed_brlen[t][a] = node.edge_length if node is not None else None
        st['fixed_brlen'] = fixed_brlen
        st['nodes_to_recompute'] = recompute
        return st

    @staticmethod
    def _swap(u, v, u_child, w):
        u_child.set_parent(v)
        u.remove_child(u_child)
        v.add_child(u_child)
        w.set_parent(u)
        v.remove_child(w)
        u.add_child(w)

    @staticmethod
    def _unswap(u, v, u_child, w):
        u_child.set_parent(u)
        v.remove_child(u_child)
        u.add_child(u_child)
        w.set_parent(v)
        u.remove_child(w)
        v.add_child(w)

    def single_nni(self, curr_score, nni_iter, strategy, only_marked=False, verbose=False):
        branches = self._branches(only_marked)
        took, score, n_attempts = False, -float("inf"), 0
        while not took and branches:
            u = branches.pop()
            took, score = self.apply_nni(u, curr_score, nni_iter, strategy)
            n_attempts += 2
        return score, n_attempts, took

    def apply_nni(self, u, curr_score, nni_iter, strategy):
        v = u.get_parent()
        w = next(x for x in v.child_nodes() if x is not u)
        u_children = u.child_nodes()
        _random.shuffle(u_children)
        st = self._local_strategy(u, v, strategy)
        for u_child in u_children:
            self._swap(u, v, u_child, w)
            s = self.solver([t.newick() for t in self.treeList_obj], self.data, self.prior,
                            self.params)
            new_score, status = s.score_tree(strategy=st)
            if status != "optimal" and strategy['local_brlen_opt']:
                st2 = deepcopy(st)
                st2['fixed_brlen'] = None
                st2['nodes_to_recompute'] = None
                s = self.solver([t.newick() for t in self.treeList_obj], self.data,
                                self.prior, self.params)
                new_score, status = s.score_tree(strategy=st2)
            if self.__accept_proposal__(curr_score, new_score, nni_iter):
                self.update_from_solver(s)
                return True, new_score
            self._unswap(u, v, u_child, w)
        return False, curr_score


class Topology_search_batched(Topology_search):
    """Topology_search_parallel's listing of every NNI move, scored in device
    batches of ``batch_size`` through one batched EM."""

    def __init__(self, *a, batch_size: int = 512, group_sites: int = 8, device="cuda",
                 native: bool = True, **k):
        super().__init__(*a, **k)
        self.batch_size = batch_size
        self.group_sites = group_sites
        self.device = device
        self.native = native   # False: one newick per candidate, as the reference lists them

    def list_all_nni(self, strategy, only_marked=False):
        fast = self._list_all_nni_native(strategy, only_marked)
        if fast is not None:
            return fast
        moves = []
        for u in self._branches(only_marked):
            v = u.get_parent()
            w = next(x for x in v.child_nodes() if x is not u)
            u_children = u.child_nodes()
            st = self._local_strategy(u, v, strategy)
            _random.shuffle(u_children)
            for u_child in u_children:
                self._swap(u, v, u_child, w)
                moves.append(([t.newick() for t in self.treeList_obj], st, (u, v, u_child, w)))
                self._unswap(u, v, u_child, w)
        return moves

    def _list_all_nni_native(self, strategy, only_marked):
        """list_all_nni for one tree with the leaf order given: the same moves
        in the same order with the same random draws, the candidates built by
        laml_nni_candidates instead of a newick per move.  The tree object
        gets the child orders each swap-and-undo of the reference's listing
        leaves (Topology_search_parallel.py:114-129) as the moves are taken,
        so every u.child_nodes() copy that is shuffled reads as it would
        there.  The strategy keeps what the batched fastEM scorer reads:
        fastEM fixes every branch whenever fixed_brlen is given
        (fastEM_solver.py:310-316), so its leaf-anchored contents are not
        built.  Returns None when the newick path must run."""
        from .encoding import encode_newick, nni_candidates
        lo = self.data.get("ordered_leaf_labels")
        if not self.native or len(self.treeList_obj) != 1 or not lo:
            return None
        tree = self.treeList_obj[0]
        leaf_order = list(lo[0])
        leaf_index = {c: i for i, c in enumerate(leaf_order)}
        ids = encoded_ids(tree, leaf_index)
        if ids is None:
            return None
        start = encode_newick(tree.newick(), leaf_order)
        snapshot = [(x, list(x.children)) for x in tree.traverse_preorder() if x.children]
        meta, pairs, sts = [], [], []
        for u in self._branches(only_marked):
            v = u.get_parent()
            w = next(x for x in v.child_nodes() if x is not u)
            st = deepcopy(strategy)
            st['fixed_brlen'] = None
            st['nodes_to_recompute'] = None
            if strategy['local_brlen_opt']:
                st['fixed_nu'] = self.params['nu']
                st['fixed_phi'] = self.params['phi']
                st['fixed_brlen'] = [{}]   # set: fastEM then fixes every branch
            u_children = u.child_nodes()
            _random.shuffle(u_children)
            for u_child in u_children:
                meta.append((u, v, u_child, w))
                pairs.append((ids[id(u)], ids[id(u_child)]))
                sts.append(st)
                keep = next(x for x in u.children if x is not u_child)
                u.children = [keep, u_child]   # what the swap and its undo leave
                v.children = [u, w]
        if not pairs:
            return []
        cands = nni_candidates(start, pairs)
        final = [(x, list(x.children)) for x, _ in snapshot]

        def newick_of(m):
            # the tree object as it read when move m was listed, swapped
            for x, ch in snapshot:
                x.children = list(ch)
            for (u, v, uc, w) in meta[:m]:
                u.children = [next(x for x in u.children if x is not uc), uc]
                v.children = [u, w]
            u, v, uc, w = meta[m]
            self._swap(u, v, uc, w)
            nw = tree.newick()
            self._unswap(u, v, uc, w)
            for x, ch in final:
                x.children = list(ch)
            return [nw]
        return [(None, st, mv, cand, (lambda m=m: newick_of(m)))
                for m, (st, mv, cand) in enumerate(zip(sts, meta, cands))]

    def single_nni(self, curr_score, nni_iter, strategy, only_marked=False, verbose=False):
        from .fastEM_solver import score_candidate_batch
        moves = self.list_all_nni(strategy, only_marked=only_marked)
        checked = 0
        for start in range(0, len(moves), self.batch_size):
            chunk = moves[start:start + self.batch_size]
            native = len(chunk) > 0 and chunk[0][0] is None
            extra = {"trees": [m[3] for m in chunk]} if native else {}
            results = score_candidate_batch(
                [m[4] if native else m[0] for m in chunk], [m[1] for m in chunk], self.data,
                self.prior, self.params, group_sites=self.group_sites, device=self.device,
                **extra)
            for res in results:
                checked += 1
                if self.__accept_proposal__(curr_score, res.score, nni_iter):
                    self.treeTopoList = res.newicks
                    self.params = res.params
                    self.__renew_treeList_obj__()
                    return res.score, checked, True
        return curr_score, checked, False
