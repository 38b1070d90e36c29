"""One tree's EM with its sites split across ranks (one process per GPU).

Sites are independent through the inside and outside passes: the reference
carries them on the leading axis of every array of the E-step
(fast_em/calculations.py:506-577).  The M-step reads only sums over sites --
the log-likelihood, the six expected transition counts of every branch and
the leaves' silencing responsibilities (fast_em/laml.py:62-78,
laml_libs/EM_solver.py:307-459).  So each rank runs the inside and outside
passes on its share of the sites, and one all-reduce per EM iteration of
8 N + 1 FP64 values (per node: the six counts and the two leaf
responsibilities; the log-likelihood) feeds an M-step that every rank runs on
the same sums: the parameters stay identical on every rank with no
broadcast.  A second all-reduce of one value carries the log-likelihood after
the M-step to the stopping rule.

This is the split for one tree too large for the per-tree sharding of
``shard.py`` to help (a 50,000-leaf tree is one unit of work there).

The reduction is host code over torch.distributed: NCCL on device tensors,
gloo through host copies.  The M-step takes the reduced counts in group 0 of
the batch's count partials (the other groups zeroed) and the whole tree's
'?' and site counts through ``laml_batch.tr_mstats``.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence

import numpy as np
import torch
import torch.distributed as dist

from . import _native as N
from .engine import EM_STOP_COMPAT, EM_STOP_EXACT, MSTEP_ROUNDS, TreeResult
from .problem import make_batch


def site_shards(state_counts: Sequence[int], world: int) -> List[np.ndarray]:
    """Original site indices of each rank's share: sites taken largest state
    count first, each to the rank with the least state slots so far (the
    passes' work per site is proportional to its state count); each share
    sorted."""
    C_ = np.asarray(state_counts, np.int64)
    load = np.zeros(world, np.int64)
    out: List[list] = [[] for _ in range(world)]
    for c in sorted(range(len(C_)), key=lambda i: (-C_[i], i)):
        r = int(np.argmin(load))
        out[r].append(c)
        load[r] += C_[c]
    return [np.asarray(sorted(x), np.int64) for x in out]


def observed_state_counts(rows: dict, leaf_order: Sequence[str], n_sites: int) -> np.ndarray:
    """Per site, the distinct observed mutated states plus 2 (the layout's
    state count in the fastEM model)."""
    seen = [set() for _ in range(n_sites)]
    for c in leaf_order:
        for k, x in enumerate(rows[c]):
            if isinstance(x, (int, np.integer)) and x > 0:
                seen[k].add(int(x))
    return np.asarray([len(s) + 2 for s in seen], np.int64)


def sub_matrix(rows: dict, Q, sites: Sequence[int]):
    """The character matrix and priors restricted to ``sites``."""
    idx = [int(s) for s in sites]
    return {c: [v[i] for i in idx] for c, v in rows.items()}, [Q[i] for i in idx]


def pack_stats(llh: float, counts8: np.ndarray) -> np.ndarray:
    """One FP64 vector: [llh, counts8 (N x 8, row-major)]."""
    return np.concatenate([[float(llh)], np.asarray(counts8, np.float64).reshape(-1)])


def unpack_stats(v, n_nodes: int):
    v = np.asarray(v, np.float64)
    return float(v[0]), v[1:].reshape(n_nodes, 8)


def all_reduce_sum(x: torch.Tensor, group=None) -> torch.Tensor:
    """Sum over ranks: in place on the device with NCCL, through a host copy
    with gloo."""
    if dist.get_backend(group) == "nccl" or x.device.type == "cpu":
        dist.all_reduce(x, op=dist.ReduceOp.SUM, group=group)
        return x
    h = x.cpu()
    dist.all_reduce(h, op=dist.ReduceOp.SUM, group=group)
    x.copy_(h)
    return x


class SiteSplitEM:
    """The EM of one tree over this rank's ``sites`` (original indices of the
    full matrix); every rank of ``group`` holds the same tree and start
    parameters and a disjoint share of the sites."""

    def __init__(self, newick: str, rows: dict, Q, leaf_order: Sequence[str],
                 sites: Sequence[int], nu=0.5, phi=0.5, compat: bool = True, d=None,
                 mask=None, fix_nu=False, fix_phi=False, group_sites: int = 8, group=None,
                 device="cuda", clamp: Optional[bool] = None):
        self.group = group
        self.compat = compat
        sub_rows, sub_Q = sub_matrix(rows, Q, sites)
        self.b = make_batch([newick], sub_rows, sub_Q, leaf_order, compat=compat,
                            group_sites=group_sites, nu=nu, phi=phi,
                            d=None if d is None else [d],
                            mask=None if mask is None else [mask], fix_nu=[fix_nu],
                            fix_phi=[fix_phi], clamp=compat if clamp is None else clamp,
                            device=device)
        b = self.b
        self.N = b.trees[0].num_nodes
        self.NG = b.datasets[0].n_groups
        dev = b.device
        # the whole tree's '?' entries and sites, for the M-step
        tot = torch.tensor([float(b.datasets[0].n_missing), float(len(sites))],
                           dtype=torch.float64, device=dev)
        all_reduce_sum(tot, group)
        self.total_missing, self.total_sites = float(tot[0]), int(round(float(tot[1])))
        self._mstats = tot
        b.b.tr_mstats = tot.data_ptr()
        self._cnt = b.work["cnt_part"][:self.N * self.NG * 8].view(self.N, self.NG, 8)
        self.reduced_counts = None

    def _llh(self) -> float:
        t = self.b.work["tr_llh"][:1].clone()
        return float(all_reduce_sum(t, self.group).item())

    def log_likelihood(self) -> float:
        """The whole tree's log-likelihood at the current parameters."""
        self.b.branch_terms()
        self.b.inside(update_em=False)
        return self._llh()

    def e_step(self) -> float:
        """Outside pass and counts on this rank's sites, then the all-reduce:
        afterwards group 0 of the count partials holds every rank's sums.
        Needs the inside pass at the current parameters (log_likelihood or
        the previous M-step's pass).  Returns the reduced log-likelihood of
        that inside pass."""
        b = self.b
        b.outside()
        loc = torch.empty(1 + self.N * 8, dtype=torch.float64, device=b.device)
        loc[0] = b.work["tr_llh"][0]
        loc[1:] = self._cnt.to(torch.float64).sum(dim=1).reshape(-1)
        all_reduce_sum(loc, self.group)
        red = loc[1:].view(self.N, 8)
        self.reduced_counts = red
        self._cnt.zero_()
        self._cnt[:, 0, :] = red.to(torch.float32)
        return float(loc[0].item())

    def m_step(self, rounds: int = MSTEP_ROUNDS):
        self.b.mstep(rounds=rounds)

    def run(self, max_iters: int = 100000, rel_tol: Optional[float] = None,
            rounds: int = MSTEP_ROUNDS) -> TreeResult:
        """EM with the stopping rule of fast_em/laml.py:112-194 (compat) or
        EM_solver.EM_optimization (exact) on the whole tree's
        log-likelihood; a negative ``rel_tol`` runs ``max_iters`` iterations.
        compat returns the parameters from before the last M-step on
        convergence, as fast_em does."""
        tol = rel_tol if rel_tol is not None else (EM_STOP_COMPAT if self.compat
                                                    else EM_STOP_EXACT)
        b = self.b
        prev = self.log_likelihood()
        it, cur, status = 0, prev, N.TREE_MAXITER
        while it < max_iters:
            it += 1
            self.e_step()
            self.m_step(rounds)
            b.inside(update_em=False)
            cur = self._llh()
            if np.isnan(cur):
                status = N.TREE_NAN
                cur = prev
                break
            if abs(cur - prev) / abs(prev) < tol:
                status = N.TREE_CONVERGED
                break
            prev = cur
        r = b.results()[0]
        if status in (N.TREE_CONVERGED, N.TREE_NAN) and self.compat:
            prevp = b.work["tr_prev"][:2].cpu().numpy()
            d = b.work["nd_d_prev"][:self.N].cpu().numpy().copy()
            return TreeResult(float(cur), float(prevp[0]), float(prevp[1]), it, status, d)
        return TreeResult(float(cur), r.nu, r.phi, it, status, r.branch_lengths)
