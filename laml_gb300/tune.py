"""Tile-shape autotuner.

Two axes of the level kernels' tiling:

* sites per group G (8, 16 or 32): how many sites share one interleaved
  state column block, hence the width of every row access (4 G bytes per
  slot) and the number of (node, group) items per warp (32 / G).  Small G
  wastes no lanes on site padding; large G gives wider transactions and
  fewer items.
* the wide levels' kernel: per-thread row loads (0); rows copied into
  per-warp shared-memory stages by the bulk-copy engine with 8 or 16 state
  slots per stage (4 or 2 stages), each warp issuing its own copies; or
  producer/consumer warp pairs, a producer warp copying rows (8 or 16
  slots per stage) and per-site scalars for its consumer warp: how the
  state loops of the levels with more than 8192 items are fed.

``autotune`` times fused EM iterations of a sample of the batch for every
shape on the device and keeps the fastest (cached per workload shape);
``pick_group_sites`` is the no-GPU cost model used when the batch is too
small for timing to mean anything.  This replaces the reference's one dense
layout: every site padded to the largest state count (fast_em/laml.py:205).
"""
from __future__ import annotations

import time
from typing import Dict, Optional, Sequence

import numpy as np

GROUP_SITES = (8, 16, 32)
# (state slots per stage, producer/consumer pairs)
WIDE_KERNELS = ((0, False), (8, False), (16, False), (8, True), (16, True))
_CACHE: Dict[tuple, dict] = {}


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


def _key(newicks, Q, compat, sample):
    n = len(newicks)
    avg = int(np.mean([s.count(",") + 1 for s in newicks[:min(n, 8)]]))
    return (min(n, sample), len(Q), avg, bool(compat))


def autotune(newicks: Sequence[str], rows, Q, leaf_order, compat=True, sample=128, iters=2,
             device="cuda", group_sites=GROUP_SITES, wide_kernels=WIDE_KERNELS) -> dict:
    """Time ``iters`` EM iterations (the graph of per-level launches, as the
    solver replays it) on the first ``sample`` trees for every (G, wide
    kernel) and return {"group_sites", "wide_chunk", "wide_pc", "ms":
    {"G/chunk" or "G/pc chunk": ms}}.  Cached per (sample size, sites, tree
    size, model)."""
    import torch

    from .problem import make_batch
    key = _key(newicks, Q, compat, sample)
    if key in _CACHE:
        return _CACHE[key]
    nw = list(newicks[:sample])
    times = {}
    best, best_t = None, None
    for G in group_sites:
        b = make_batch(nw, rows, Q, leaf_order, compat=compat, group_sites=G, device=device)
        for ch, pc in wide_kernels:
            b.wide_chunk = ch
            b.wide_pc = pc
            b.branch_terms()
            b.inside(update_em=True)
            g = b.em_graph(iters, rel_tol=-1.0, max_iters=1 << 30, persistent=False)
            b.launch_graph(g)   # warm
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b.launch_graph(g)
            torch.cuda.synchronize()
            t = (time.perf_counter() - t0) / iters
            times[f"{G}/pc {ch}" if pc else f"{G}/{ch}"] = t * 1e3
            if best_t is None or t < best_t:
                best, best_t = (G, ch, pc), t
        del b
    out = {"group_sites": best[0], "wide_chunk": best[1], "wide_pc": best[2], "ms": times,
           "sample_trees": len(nw), "iters": iters}
    _CACHE[key] = out
    return out
