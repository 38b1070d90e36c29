"""Public batched entry points.

``score_candidates`` scores many candidate topologies over one character
matrix in one device batch -- what Topology_search does one
``fastEM_solver(...).score_tree(strategy)`` at a time
(laml_libs/Topology_search.py:299-306, fastEM_solver.py:283-353): every tree
starts at nu = phi = 0.5 (fastEM_solver.py:320-321) with both free, its own
branch lengths (random U(0.01, 0.5) where missing, fastEM_solver.py:95-126),
and runs fastEM's EM to its stopping rule; the score is the final
log-likelihood.
"""
from __future__ import annotations

import random
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np
import torch

from .engine import MSTEP_ROUNDS, TreeResult
from .encoding import encode_newick_batch
from .problem import dataset_from_rows, make_batch


@dataclass
class ScoreResult:
    results: List[TreeResult]
    h2d_bytes: int
    d2h_bytes: int

    @property
    def scores(self):
        return [r.llh for r in self.results]


def score_candidates(newicks: Sequence[str], rows: dict, Q, leaf_order: Sequence[str],
                     compat: bool = True, group_sites: int = 8, nu: float = 0.5,
                     phi: float = 0.5, rounds: int = MSTEP_ROUNDS, max_iters: int = 100000,
                     fix_nu=None, fix_phi=None, masks=None, device="cuda", chunk: int = 4,
                     rng: Optional[random.Random] = None) -> ScoreResult:
    ds = dataset_from_rows(rows, Q, leaf_order, compat, group_sites)
    trees = encode_newick_batch(newicks, leaf_order)
    rng = rng if rng is not None else random
    d = []
    for t in trees:
        x = t.branch_length.copy()
        if not t.has_length.all():
            # fastEM_solver.parse_tree draws U(0.01, 0.5): leaves first, then internal nodes
            for i in np.flatnonzero(~t.has_length):
                x[i] = rng.uniform(0.01, 0.5)
        d.append(x)
    b = make_batch(newicks, rows, Q, leaf_order, compat=compat, group_sites=group_sites, nu=nu,
                   phi=phi, d=d, mask=masks, fix_nu=fix_nu, fix_phi=fix_phi, device=device,
                   trees=trees, dataset=ds)
    res = b.run_em(rounds=rounds, max_iters=max_iters, chunk=chunk)
    d2h = b.last_d2h_bytes
    return ScoreResult(res, b.h2d_bytes, d2h)
