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
import threading
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


def part_bounds(T: int, parts: int) -> List[int]:
    """Bounds of the pipeline parts of T candidates: part k holds a share
    k + 1, so the first part's host work -- the only host work not hidden
    behind a part's EM -- is the smallest."""
    wsum = parts * (parts + 1) // 2
    return [T * (k * (k + 1) // 2) // wsum for k in range(parts + 1)]


_STREAMS: dict = {}
_STREAMS_LOCK = threading.Lock()


def _part_stream(dev, k):
    """The stream of pipeline part k on a device, the same across calls: the
    caching allocator keeps freed device blocks per stream, so a part that
    reuses its stream reuses the previous call's buffers instead of
    allocating afresh."""
    with _STREAMS_LOCK:
        key = (str(dev), k)
        if key not in _STREAMS:
            _STREAMS[key] = torch.cuda.Stream(dev)
        return _STREAMS[key]


def score_candidates(newicks: Sequence[str], rows: dict, Q, leaf_order: Sequence[str],
                     compat: bool = True, group_sites: Optional[int] = None,
                     wide_chunk: Optional[int] = None, wide_pc: Optional[bool] = None,
                     nu: float = 0.5,
                     phi: float = 0.5, rounds: int = MSTEP_ROUNDS, max_iters: int = 100000,
                     fix_nu=None, fix_phi=None, masks=None, device="cuda", chunk: int = 4,
                     rng: Optional[random.Random] = None,
                     pipeline: Optional[int] = None) -> ScoreResult:
    """``pipeline`` parts: the candidates are cut into that many contiguous
    parts of growing size (part k holds a share k + 1), each its own device
    batch on its own stream; a worker thread parses, plans and uploads part
    k+1 while part k iterates, so the host work of all parts but the first
    -- the smallest -- overlaps the device, and the matrix is encoded on a
    second thread while the first part's newicks are parsed.  Each part's EM
    (one launch of its EM loop graph) goes to the device as soon as the part
    is built and runs beside the parts queued before it; the results are
    collected at the end.  Each tree's EM is
    independent of the others in its batch, so the parts give each tree the
    result it has in one batch (up to FP32 summation order when a level's
    width crosses the wide/narrow rule).  Default: 2 parts from 256
    candidates on, else 1.

    ``group_sites`` / ``wide_chunk`` / ``wide_pc`` (the tile shape and the
    wide levels' kernel): None = picked by the autotuner (``tune.autotune``,
    cached per workload shape) for 64 or more candidates, by the cost model
    below that."""
    import threading
    from concurrent.futures import ThreadPoolExecutor

    from . import tune

    if group_sites is None or wide_chunk is None or wide_pc is None:
        if len(newicks) >= 64 and torch.device(device).type == "cuda":
            t = tune.autotune(newicks, rows, Q, leaf_order, compat=compat, device=device)
        else:
            t = {"group_sites": tune.pick_group_sites(n_sites=len(Q)), "wide_chunk": 0,
                 "wide_pc": False}
        group_sites = t["group_sites"] if group_sites is None else group_sites
        wide_chunk = t["wide_chunk"] if wide_chunk is None else wide_chunk
        wide_pc = bool(t.get("wide_pc", False)) if wide_pc is None else wide_pc
    rng = rng if rng is not None else random
    T = len(newicks)
    parts = pipeline if pipeline is not None else (2 if T >= 256 else 1)
    parts = max(1, min(int(parts), T))
    bounds = part_bounds(T, parts)
    ds_pool = ThreadPoolExecutor(1)
    # the matrix encodes while the first part's newicks are parsed
    ds_fut = ds_pool.submit(dataset_from_rows, rows, Q, leaf_order, compat, group_sites)
    dev = torch.device(device)
    if dev.type == "cuda" and dev.index is None:   # the worker thread needs the index
        dev = torch.device("cuda", torch.cuda.current_device())

    def prep(k):
        lo, hi = bounds[k], bounds[k + 1]
        nws = list(newicks[lo:hi])
        trees = encode_newick_batch(nws, leaf_order)
        d = []
        for t in trees:
            x = t.branch_length.copy()
            if not t.has_length.all():
                # fastEM_solver.parse_tree draws U(0.01, 0.5): leaves first, then internal nodes
                for i in np.flatnonzero(~t.has_length):
                    x[i] = rng.uniform(0.01, 0.5)
            d.append(x)
        ds = ds_fut.result()
        sub = lambda a: None if a is None else (a[lo:hi] if not np.isscalar(a) else a)  # noqa: E731
        if dev.type == "cuda" and threading.current_thread() is not threading.main_thread():
            torch.cuda.set_device(dev)
        st = _part_stream(dev, k) if (parts > 1 and dev.type == "cuda") else None
        b = make_batch(nws, rows, Q, leaf_order, compat=compat, group_sites=group_sites, nu=nu,
                       phi=phi, d=d, mask=sub(masks), fix_nu=sub(fix_nu), fix_phi=sub(fix_phi),
                       device=device, trees=trees, dataset=ds, stream=st)
        b.wide_chunk = wide_chunk
        b.wide_pc = wide_pc
        return b, st

    res, h2d, d2h = [], 0, 0
    if parts == 1:
        b, _ = prep(0)
        ds_pool.shutdown()
        res = b.run_em(rounds=rounds, max_iters=max_iters, chunk=chunk)
        return ScoreResult(res, b.h2d_bytes, b.last_d2h_bytes)
    with ThreadPoolExecutor(1) as ex:
        fut = ex.submit(prep, 0)
        queued = []
        for k in range(parts):
            b, st = fut.result()
            if k + 1 < parts:
                fut = ex.submit(prep, k + 1)
            # each part's EM goes to the device as soon as the part is built,
            # on its own stream, and runs beside the parts queued before it
            with torch.cuda.stream(st):
                b.run_em_start(rounds=rounds, max_iters=max_iters, chunk=chunk)
            queued.append((b, st))
        for b, st in queued:
            with torch.cuda.stream(st):
                res += b.run_em_finish()
            h2d += b.h2d_bytes
            d2h += b.last_d2h_bytes
        del queued
    ds_pool.shutdown()
    return ScoreResult(res, h2d, d2h)
