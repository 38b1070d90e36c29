"""Tile-shape autotuner: sites per warp group (G = 8, 16 or 32).

G sets how many sites share one interleaved state column block, hence the
coalescing width of every load (4*G bytes per group) and the number of
(node, group) items per warp (32/G).  Small G wastes no lanes on site
padding; large G gives wider transactions.  ``autotune`` times a few fused
EM iterations of a sub-batch for each G on the device and keeps the fastest;
``pick_group_sites`` is the no-GPU fallback cost model.
"""
from __future__ import annotations

import time
from typing import Dict, Optional, Sequence

import numpy as np

_CACHE: Dict[tuple, int] = {}


def _padding_cost(K: int, G: int) -> float:
    Kp = (K + G - 1) // G * G
    return Kp / K


def pick_group_sites(workload=None, n_sites: Optional[int] = None) -> int:
    """Cost model: the smallest G whose site padding wastes under 12.5% of
    lanes, preferring wider groups (coalescing) when padding is equal."""
    K = n_sites if n_sites is not None else len(workload.Q)
    best, best_cost = 8, None
    for G in (32, 16, 8):
        waste = _padding_cost(K, G) - 1.0
        cost = waste + {32: 0.0, 16: 0.04, 8: 0.08}[G]
        if best_cost is None or cost < best_cost:
            best, best_cost = G, cost
    return best


def autotune(newicks: Sequence[str], rows, Q, leaf_order, compat=True, sample=32, iters=3,
             device="cuda") -> int:
    """Time ``iters`` fused EM iterations on ``sample`` trees for each G."""
    import torch

    from .problem import make_batch
    key = (len(newicks), len(Q), compat)
    if key in _CACHE:
        return _CACHE[key]
    nw = list(newicks[:sample])
    best, best_t = 8, None
    for G in (8, 16, 32):
        b = make_batch(nw, rows, Q, leaf_order, compat=compat, group_sites=G, device=device)
        b.branch_terms()
        b.inside(update_em=True)
        b.em_iterations(1, rel_tol=-1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.em_iterations(iters, rel_tol=-1.0)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        if best_t is None or t < best_t:
            best, best_t = G, t
        del b
    _CACHE[key] = best
    return best
