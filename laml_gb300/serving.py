"""Continuous-batching server for PMM likelihood / EM requests.

Requests (a tree, its character matrix and priors, a kind -- "llh" for one
log-likelihood, "em" for fastEM's EM to convergence -- and starting nu, phi)
are encoded on the submitting thread (C++ encoders) and queued.  A scheduler
thread admits queued requests into *cohorts* whenever cohort slots and HBM
budget are free: a cohort is one DeviceBatch (any mix of tree sizes and
site counts) on its own CUDA stream, driven in chunks of fused EM iterations
with per-level launches, so cohorts admitted at different times run
concurrently on the device.  Encoded inputs, partials and EM state stay on
the GPU; a request's future resolves as soon as its own tree leaves the
ACTIVE state.

Continuous batching at iteration boundaries: when a chunk of an EM cohort
ends with some of its trees finished, the cohort is rebuilt from its
unfinished trees -- each carrying its EM state (branch lengths, nu, phi, the
log-likelihood the stopping rule compares against, its iteration count) --
joined by queued EM requests that fit the memory the finished trees leave.
The finished trees' memory returns to the budget then, and new arrivals
start at the next iteration boundary instead of waiting for a whole cohort.

Each tree's arithmetic does not depend on what else is in its batch, so a
request's result is the same alone or in any mix: bitwise while its levels
fall on the same side of the narrow / wide rule (a level with more than 8192
items of the batch runs the per-thread kernels), else to FP32 summation
order.
"""
from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np
import torch

from . import _native as N
from .encoding import EncodedDataset, EncodedTree, char_matrix, encode_dataset, encode_newick
from .encoding import plan_batch
from .engine import MSTEP_ROUNDS, DeviceBatch, TreeResult

EPS = 1e-6


@dataclass
class Request:
    newick: str
    rows: Dict[str, list]
    Q: List[dict]
    leaf_order: Optional[List[str]] = None
    kind: str = "em"              # "llh" or "em"
    nu: float = 0.5
    phi: float = 0.5
    # the matrix already encoded (PMMServer.encode_dataset): a client that
    # scores many trees against one matrix -- topology-search candidates --
    # encodes it once instead of with every request
    dataset: Optional[EncodedDataset] = None


@dataclass
class Reply:
    result: TreeResult
    t_submit: float
    t_admit: float
    t_done: float

    @property
    def latency(self):
        return self.t_done - self.t_submit


# the server's own records compare by identity: their fields hold arrays,
# and a list of them is searched with == (list.remove, in)
@dataclass(eq=False)
class _Job:
    req: Request
    tree: EncodedTree
    ds: EncodedDataset
    footprint: int
    future: Future
    t_submit: float
    t_admit: float = 0.0


@dataclass(eq=False)
class _Cohort:
    jobs: List[_Job]
    batch: DeviceBatch
    stream: torch.cuda.Stream
    kind: str
    footprint: int
    event: torch.cuda.Event
    done: np.ndarray = None
    host_status: torch.Tensor = None


def footprint_bytes(tree: EncodedTree, ds: EncodedDataset) -> int:
    """Device bytes a single-tree batch of this request holds."""
    sizes, _ = plan_batch([tree], [0], [ds], host_desc=False)
    nn = sizes["n_nodes"]
    return int(8 * sizes["part_floats"] + 20 * sizes["scalar_len"] + 4 * sizes["count_floats"]
               + 200 * nn + ds.codes.nbytes + 4 * ds.row_len + 64 * ds.n_sites_pad
               + 56 * sizes["n_in_items"] + 56 * sizes["n_out_items"])


class PMMServer:
    def __init__(self, device="cuda", hbm_budget: int = 64 << 30, max_cohort: int = 256,
                 max_cohorts: int = 6, group_sites: int = 8, rounds: int = MSTEP_ROUNDS,
                 chunk: int = 4, max_iters: int = 1000, max_em_cohort: int = 128,
                 graphs: bool = True):
        self.device = torch.device(device)
        self.budget = hbm_budget
        self.max_cohort = max_cohort
        self.max_em_cohort = max_em_cohort   # EM cohorts smaller: a slow tree holds its cohort
        self.max_cohorts = max_cohorts
        # tree-EM-iterations launched (counted when each chunk is queued) and
        # those of the requests answered (counted from their results)
        self.em_tree_iterations = 0
        self.em_tree_iterations_completed = 0
        self.recohorts = 0
        self.G = group_sites
        self.rounds = rounds
        self.chunk = chunk
        self.graphs = graphs   # EM chunks as graph replays (else per-level launches)
        # fastEM's loop has no cap (fast_em/laml.py:153: while True) and some
        # problems alternate between two log-likelihoods further apart than
        # its 1e-5 rule forever; a request stops after max_iters iterations
        # (EM_solver's own cap, 1000) with status LAML_TREE_MAXITER
        self.max_iters = max_iters
        self._pending: collections.deque = collections.deque()
        self._lock = threading.Lock()
        self._wake = threading.Event()
        self._active: List[_Cohort] = []
        self._used = 0
        self._closing = False
        self._abort = False
        self._streams = [torch.cuda.Stream(self.device) for _ in range(max_cohorts)]
        self._free_streams = list(self._streams)
        self.error: Optional[BaseException] = None
        self._thread = threading.Thread(target=self._run, daemon=True)
        self._thread.start()

    # -- client side ------------------------------------------------------
    def encode_dataset(self, rows: Dict[str, list], Q: List[dict],
                       leaf_order: List[str]) -> EncodedDataset:
        """The site layout of a matrix, for Request.dataset."""
        return encode_dataset(char_matrix([rows[c] for c in leaf_order]), Q, compat=True,
                              group_sites=self.G)

    def submit(self, req: Request) -> Future:
        t0 = time.perf_counter()
        lo = req.leaf_order
        tree = encode_newick(req.newick, lo)
        if req.dataset is not None:
            if req.dataset.group_sites != self.G or req.dataset.n_leaves != tree.num_leaves:
                raise ValueError("Request.dataset does not match the server or the tree")
            ds = req.dataset
        else:
            order = lo if lo is not None else tree.labels[:tree.num_leaves]
            ds = encode_dataset(char_matrix([req.rows[c] for c in order]), req.Q, compat=True,
                                group_sites=self.G)
        fp = footprint_bytes(tree, ds)
        if fp > self.budget:
            raise ValueError(f"request needs {fp} bytes of HBM, the budget is {self.budget}")
        fut: Future = Future()
        with self._lock:
            self._pending.append(_Job(req, tree, ds, fp, fut, t0))
        self._wake.set()
        return fut

    def snapshot(self):
        """The EM requests on the device now: leaves, sites, EM iterations
        done and seconds since submission (reads the iteration counters:
        a synchronising copy per cohort)."""
        out = []
        now = time.perf_counter()
        for c in list(self._active):
            if c.kind != "em" or c.batch is None:
                continue
            with torch.cuda.stream(c.stream):
                it = c.batch.work["tr_iter"].cpu().numpy()
                llh = c.batch.work["tr_llh"].cpu().numpy()
            for i, j in enumerate(c.jobs):
                if not c.done[i]:
                    out.append({"leaves": int(j.tree.num_leaves), "sites": int(j.ds.n_sites),
                                "iterations": int(it[i]), "llh": float(llh[i]),
                                "seconds": now - j.t_submit})
        return out

    def close(self, wait: bool = True):
        """Stop the server.  wait=True: finish every submitted request first;
        wait=False: launch no further work and fail the requests not yet
        answered (work already queued on the GPU finishes on its own)."""
        self._closing = True
        if not wait:
            self._abort = True
        self._wake.set()
        self._thread.join()
        if self.error is not None:
            raise self.error

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
        return False

    # -- scheduler ----------------------------------------------------------
    def _admit(self):
        while self._free_streams:
            with self._lock:
                if not self._pending:
                    return
                # log-likelihood requests (one inside pass) go first; EM
                # cohorts -- dozens of iterations each -- leave one stream
                # free for them, so a burst of EM work cannot starve them
                kinds = {j.req.kind for j in self._pending}
                if "llh" in kinds:
                    kind = "llh"
                elif len(self._free_streams) > 1 or self.max_cohorts == 1:
                    kind = "em"
                else:
                    return
                jobs, used = [], 0
                rest = collections.deque()
                cap = self.max_cohort if kind == "llh" else self.max_em_cohort
                while self._pending and len(jobs) < cap:
                    j = self._pending.popleft()
                    if j.req.kind == kind and self._used + used + j.footprint <= self.budget:
                        jobs.append(j)
                        used += j.footprint
                    else:
                        rest.append(j)
                        if j.req.kind == kind:
                            break          # FIFO within a kind: wait for memory
                rest.extend(self._pending)
                self._pending = rest
            if not jobs:
                return
            self._used += used
            self._launch(jobs, kind, used)

    def _launch(self, jobs: List[_Job], kind: str, used: int):
        stream = self._free_streams.pop()
        now = time.perf_counter()
        for j in jobs:
            j.t_admit = now
        with torch.cuda.stream(stream):
            nu = np.clip([j.req.nu for j in jobs], EPS, 1 - EPS)
            phi = np.clip([j.req.phi for j in jobs], EPS, 1 - EPS)
            d = [np.maximum(j.tree.branch_length, EPS) for j in jobs]
            # one copy of each distinct encoded matrix in the cohort
            uniq, tree_ds = {}, []
            for j in jobs:
                tree_ds.append(uniq.setdefault(id(j.ds), (len(uniq), j.ds))[0])
            dsets = [x for _, x in sorted(uniq.values(), key=lambda t: t[0])]
            b = DeviceBatch(dsets, [j.tree for j in jobs], tree_ds, d, nu, phi, compat=True,
                            device=self.device, stream=stream)
            b.branch_terms()
            b.inside(update_em=True)
            if kind == "em":
                self._em_chunk(b)
                self.em_tree_iterations += self.chunk * len(jobs)
            host = torch.empty(len(jobs), dtype=torch.int32, pin_memory=True)
            host.copy_(b.work["tr_status"], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        c = _Cohort(jobs, b, stream, kind, used, ev, np.zeros(len(jobs), bool), host)
        self._active.append(c)

    def _progress(self, c: _Cohort) -> bool:
        """Returns True when the cohort is finished."""
        if not c.event.query():
            return False
        b = c.batch
        now = time.perf_counter()
        if c.kind == "llh":
            with torch.cuda.stream(c.stream):
                llh = b.work["tr_llh"].cpu().numpy()
            for i, j in enumerate(c.jobs):
                r = TreeResult(float(llh[i]), float(j.req.nu), float(j.req.phi), 0,
                               N.TREE_CONVERGED, j.tree.branch_length.copy())
                j.future.set_result(Reply(r, j.t_submit, j.t_admit, now))
            return True
        st = c.host_status.numpy()
        newly = (~c.done) & (st != N.TREE_ACTIVE)
        if newly.any():
            with torch.cuda.stream(c.stream):
                res = b.results()
            for i in np.flatnonzero(newly):
                j = c.jobs[i]
                self.em_tree_iterations_completed += int(res[i].iterations)
                j.future.set_result(Reply(res[i], j.t_submit, j.t_admit, now))
            c.done |= newly
        if c.done.all():
            return True
        if c.done.any():
            c = self._recohort(c)
            b = c.batch
        with torch.cuda.stream(c.stream):
            self._em_chunk(b)
            self.em_tree_iterations += self.chunk * int((~c.done).sum())
            c.host_status.copy_(b.work["tr_status"], non_blocking=True)
            c.event.record(c.stream)
        return False

    def _em_chunk(self, b: DeviceBatch):
        """One chunk of EM iterations on a cohort: a replay of the cohort
        batch's CUDA graph (captured on its first chunk), one launch instead
        of ~50 per iteration from the server thread."""
        if self.graphs:
            b.launch_graph(b.em_graph(self.chunk, rounds=self.rounds, max_iters=self.max_iters,
                                      persistent=False))
        else:
            b.em_iterations(self.chunk, rounds=self.rounds, max_iters=self.max_iters,
                            persistent=False)

    def _recohort(self, c: _Cohort) -> _Cohort:
        """Rebuild an EM cohort at an iteration boundary from its unfinished
        trees (EM state carried over) and the queued EM requests that fit the
        memory its finished trees free; the old batch is released."""
        b = c.batch
        keep = [i for i in range(len(c.jobs)) if not c.done[i]]
        with torch.cuda.stream(c.stream):
            res = b.results()
            prev = b.work["tr_llh_prev"].cpu().numpy()
            iters = b.work["tr_iter"].cpu().numpy()
        kept = [c.jobs[i] for i in keep]
        used = sum(j.footprint for j in kept)
        add = []
        with self._lock:
            rest = collections.deque()
            while self._pending and len(kept) + len(add) < self.max_em_cohort:
                j = self._pending.popleft()
                if j.req.kind == "em" and self._used - c.footprint + used + j.footprint <= self.budget:
                    add.append(j)
                    used += j.footprint
                else:
                    rest.append(j)
                    if j.req.kind == "em":
                        break
            rest.extend(self._pending)
            self._pending = rest
        now = time.perf_counter()
        for j in add:
            j.t_admit = now
        jobs = kept + add
        d = [res[i].branch_lengths for i in keep] + \
            [np.maximum(j.tree.branch_length, EPS) for j in add]
        nu = [res[i].nu for i in keep] + [min(max(j.req.nu, EPS), 1 - EPS) for j in add]
        phi = [res[i].phi for i in keep] + [min(max(j.req.phi, EPS), 1 - EPS) for j in add]
        with torch.cuda.stream(c.stream):
            uniq, tree_ds = {}, []
            for j in jobs:
                tree_ds.append(uniq.setdefault(id(j.ds), (len(uniq), j.ds))[0])
            dsets = [x for _, x in sorted(uniq.values(), key=lambda t: t[0])]
            nb = DeviceBatch(dsets, [j.tree for j in jobs], tree_ds, d, nu, phi, compat=True,
                             device=self.device, stream=c.stream)
            nb.branch_terms()
            nb.inside(update_em=True)
            k = len(keep)
            if k:   # the kept trees' stopping-rule state
                nb.work["tr_llh_prev"][:k].copy_(torch.from_numpy(prev[keep]))
                nb.work["tr_llh"][:k].copy_(torch.from_numpy(prev[keep]))
                nb.work["tr_iter"][:k].copy_(torch.from_numpy(iters[keep]))
        self._used += used - c.footprint
        self.recohorts += 1
        return _replace_cohort(self._active, c, _Cohort(
            jobs, nb, c.stream, "em", used, c.event, np.zeros(len(jobs), bool),
            torch.empty(len(jobs), dtype=torch.int32, pin_memory=True)))

    def _run(self):
        try:
            while True:
                if self._abort:
                    gone = RuntimeError("server closed before the request finished")
                    with self._lock:
                        for j in self._pending:
                            j.future.set_exception(gone)
                        self._pending.clear()
                    for c in self._active:
                        for j in c.jobs:
                            if not j.future.done():
                                j.future.set_exception(gone)
                    return
                self._admit()
                finished = [c for c in self._active if self._progress(c)]
                for c in finished:
                    self._active.remove(c)
                    self._used -= c.footprint
                    self._free_streams.append(c.stream)
                    c.batch = None
                with self._lock:
                    idle = not self._pending and not self._active
                if idle and self._closing:
                    return
                if not finished:
                    self._wake.wait(0.0002)
                    self._wake.clear()
        except BaseException as ex:   # surface to every waiter
            self.error = ex
            with self._lock:
                for j in self._pending:
                    j.future.set_exception(ex)
            for c in self._active:
                for j in c.jobs:
                    if not j.future.done():
                        j.future.set_exception(ex)


def _replace_cohort(active: List[_Cohort], old: _Cohort, new: _Cohort) -> _Cohort:
    active[next(i for i, x in enumerate(active) if x is old)] = new
    return new


def run_alone(req: Request, group_sites: int = 8, rounds: int = MSTEP_ROUNDS,
              device="cuda", max_iters: int = 1000) -> TreeResult:
    """The same request outside the server (for mix-vs-alone checks)."""
    lo = req.leaf_order
    tree = encode_newick(req.newick, lo)
    order = lo if lo is not None else tree.labels[:tree.num_leaves]
    ds = encode_dataset(char_matrix([req.rows[c] for c in order]), req.Q, compat=True,
                        group_sites=group_sites)
    b = DeviceBatch([ds], [tree], [0], [np.maximum(tree.branch_length, EPS)],
                    [min(max(req.nu, EPS), 1 - EPS)], [min(max(req.phi, EPS), 1 - EPS)],
                    compat=True, device=device)
    if req.kind == "llh":
        llh = float(b.log_likelihood()[0])
        return TreeResult(llh, req.nu, req.phi, 0, N.TREE_CONVERGED, tree.branch_length.copy())
    return b.run_em(rounds=rounds, persistent=False, max_iters=max_iters)[0]
