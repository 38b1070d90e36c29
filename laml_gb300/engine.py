"""Device-resident batch of PMM problems and the calls that run on it.

A ``DeviceBatch`` holds, in HBM, one or more encoded datasets (character
matrix + priors in the site layout), any number of trees over them, their
parameters, the inside/outside partials and the EM state.  Every compute call
goes through the C ABI of liblaml_gb300.so (laml_inside, laml_outside,
laml_mstep, laml_em_run, ...); torch is used only to own device memory and
streams.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native as N
from .encoding import EncodedDataset, EncodedTree, plan_batch

EM_STOP_COMPAT = 1e-5    # fast_em/laml.py:46
EM_STOP_EXACT = 1e-8     # laml_libs/core_constants.py:5 (conv_eps)
MSTEP_ROUNDS = 4


class _Packer:
    """Packs many small host arrays into one pinned buffer per call so a batch
    uploads with a single host->device copy."""

    ALIGN = 256

    def __init__(self):
        self.items = []
        self.size = 0

    def add(self, name, a):
        a = np.ascontiguousarray(a)
        off = (self.size + self.ALIGN - 1) // self.ALIGN * self.ALIGN
        self.items.append((name, a, off))
        self.size = off + a.nbytes
        return name

    def upload(self, device, stream=None):
        host = torch.empty(max(self.size, 1), dtype=torch.uint8, pin_memory=True)
        hv = host.numpy()
        for _, a, off in self.items:
            hv[off:off + a.nbytes] = a.view(np.uint8).reshape(-1)
        dev = torch.empty(max(self.size, 1), dtype=torch.uint8, device=device)
        dev.copy_(host, non_blocking=True)
        views = {}
        for name, a, off in self.items:
            t = torch.from_numpy(np.empty(0, a.dtype)).dtype
            views[name] = dev[off:off + a.nbytes].view(t).view(a.shape)
        return dev, host, views


@dataclass
class TreeResult:
    llh: float
    nu: float
    phi: float
    iterations: int
    status: int
    branch_lengths: np.ndarray


def ultra_schedule(trees: Sequence[EncodedTree], node_base: np.ndarray) -> np.ndarray:
    """nd_uorder of a batch: each tree's laml_ultra_order depth schedule at
    offset 2 * node_base[p] + 2 * p."""
    nn = int(sum(t.num_nodes for t in trees))
    out = np.zeros(2 * nn + 2 * len(trees), np.int32)
    w = N.i64()
    for p, t in enumerate(trees):
        o = 2 * int(node_base[p]) + 2 * p
        par = np.ascontiguousarray(t.parent, np.int32)
        N.check(N.lib().laml_ultra_order(par.ctypes.data, t.num_nodes,
                                         out[o:].ctypes.data, 2 * t.num_nodes + 2, C.byref(w)))
    return out


class DeviceBatch:
    """Trees (EncodedTree) over datasets (EncodedDataset) resident on one GPU.

    ``d``: per-tree float64 branch lengths (node order of the tree);
    ``nu``, ``phi``: per-tree starting values; ``mask``: per-tree bool arrays
    (True = branch length optimised); ``fix_nu`` / ``fix_phi``: per-tree flags;
    ``ultrametric``: exact model only -- every M-step solves the branch
    lengths under EM_solver's ultrametric equalities (EM_solver.py:53-89),
    by the primal-dual method (set the attribute ``ultra_barrier`` to use the
    log-barrier method alone).
    """

    def __init__(self, datasets: Sequence[EncodedDataset], trees: Sequence[EncodedTree],
                 tree_ds: Sequence[int], d: Sequence[np.ndarray], nu, phi, compat: bool = True,
                 mask: Optional[Sequence[np.ndarray]] = None, fix_nu=None, fix_phi=None,
                 want_post: bool = False, device="cuda", stream: Optional[torch.cuda.Stream] = None,
                 ultrametric: bool = False):
        G = datasets[0].group_sites
        for ds in datasets:
            if ds.group_sites != G or ds.compat != compat:
                raise ValueError("every dataset of a batch needs the same group size and mode")
        T = len(trees)
        if ultrametric and compat:
            raise ValueError("the ultrametric M-step belongs to the exact model (compat=False)")
        self.T, self.compat, self.G = T, compat, G
        self.ultrametric = bool(ultrametric)
        # select the ultrametric M-step's log-barrier method alone
        self.ultra_barrier = False
        # cap its primal-dual phase at 3 iterations (the barrier phase continues)
        self.ultra_pd_short = False
        self._lbfgs = False
        self.device = torch.device(device)
        self.stream = stream
        self.trees = list(trees)
        self.tree_ds = np.asarray(tree_ds, np.int32)
        self.datasets = list(datasets)
        sizes, plan = plan_batch(trees, tree_ds, datasets, host_desc=False, items=False)
        self.sizes = sizes
        self._node_base = plan["tr_node_base"].astype(np.int64)
        self.last_d2h_bytes = 0
        nn = sizes["n_nodes"]
        nu = np.broadcast_to(np.asarray(nu, np.float64), (T,)).copy()
        phi = np.broadcast_to(np.asarray(phi, np.float64), (T,)).copy()
        fix = np.zeros(T, np.uint8)
        if fix_nu is not None:
            fix |= np.broadcast_to(np.asarray(fix_nu, bool), (T,)).astype(np.uint8)
        if fix_phi is not None:
            fix |= (np.broadcast_to(np.asarray(fix_phi, bool), (T,)).astype(np.uint8) << 1)
        dcat = np.concatenate([np.asarray(x, np.float64) for x in d])
        if mask is None:
            mcat = np.ones(nn, np.uint8)
        else:
            mcat = np.concatenate([np.asarray(m, bool) for m in mask]).astype(np.uint8)
        if dcat.shape[0] != nn or mcat.shape[0] != nn:
            raise ValueError("branch lengths / masks do not match the trees")

        D = len(datasets)
        ds_sites = np.asarray([x.n_sites for x in datasets], np.int32)
        ds_kpad = np.asarray([x.n_sites_pad for x in datasets], np.int32)
        ds_groups = np.asarray([x.n_groups for x in datasets], np.int32)
        ds_site_base = np.zeros(D, np.int32)
        ds_site_base[1:] = np.cumsum(ds_kpad)[:-1]
        ds_q_base = np.zeros(D, np.int64)
        ds_q_base[1:] = np.cumsum([x.row_len for x in datasets])[:-1]
        ds_code_base = np.zeros(D, np.int64)
        ds_code_base[1:] = np.cumsum([x.codes.size for x in datasets])[:-1]

        pk = _Packer()
        for k, a in [("ds_sites", ds_sites), ("ds_sites_pad", ds_kpad), ("ds_groups", ds_groups),
                     ("ds_group_base", plan["group_base"]), ("ds_site_base", ds_site_base),
                     ("ds_q_base", ds_q_base), ("ds_code_base", ds_code_base),
                     ("ds_missing", np.asarray([x.n_missing for x in datasets], np.float64)),
                     ("ds_silenced", np.asarray([x.n_silenced for x in datasets], np.float64)),
                     ("group_off", np.concatenate([x.group_off for x in datasets])),
                     ("group_C", np.concatenate([x.group_C for x in datasets])),
                     ("site_C", np.concatenate([x.site_C for x in datasets])),
                     ("site_sumq", np.concatenate([x.site_sumq for x in datasets])),
                     ("q", np.concatenate([x.q for x in datasets])),
                     ("codes", np.concatenate([x.codes.reshape(-1) for x in datasets])),
                     ("tr_ds", self.tree_ds),
                     ("tr_nodes", np.asarray([t.num_nodes for t in trees], np.int32)),
                     ("tr_leaves", np.asarray([t.num_leaves for t in trees], np.int32)),
                     ("tr_nu", nu), ("tr_phi", phi), ("tr_fix", fix),
                     ("nd_d", dcat), ("nd_mask", mcat)]:
            pk.add(k, a)
        if ultrametric:
            pk.add("nd_uorder", ultra_schedule(trees, self._node_base))
        for k in ("tr_node_base", "tr_root", "tr_quirk", "tr_site_base", "tr_cnt_base",
                  "tr_post_base", "nd_tree", "nd_c0", "nd_c1", "nd_parent", "nd_sib",
                  "nd_leafrow", "nd_prow", "nd_srow", "in_level_off", "out_level_off",
                  "root_items", "in_items", "out_items", "in_lnodes", "out_lnodes"):
            if k in plan:   # items, or the level node lists the device expands
                pk.add(k, plan[k])
        self._h2d_bytes = pk.size
        ctx = torch.cuda.stream(stream) if stream is not None else _nullctx()
        with ctx:
            self._blob, self._pinned, v = pk.upload(self.device)
        self.v = v
        dev = self.device
        f32, f64, i32 = torch.float32, torch.float64, torch.int32
        e = lambda n, t: torch.empty(max(int(n), 1), dtype=t, device=dev)  # noqa: E731
        self.work = {
            "tr_prev": e(2 * T, f64), "tr_llh": e(T, f64), "tr_llh_prev": e(T, f64),
            "tr_iter": torch.zeros(T, dtype=i32, device=dev),
            "tr_status": torch.zeros(T, dtype=i32, device=dev),
            "tr_mode": torch.zeros(T, dtype=i32, device=dev),
            "tr_leaf": e(2 * T, f32),
            "nd_d_prev": e(nn, f64), "nd_bt": e(4 * nn, f32), "nd_cnt": e(6 * nn, f64),
            "nd_stage": e(5 * nn, f32),
            "in_part": e(sizes["part_floats"], f32), "out_part": e(sizes["part_floats"], f32),
            "in_dot": e(sizes["scalar_len"], f32), "in_x": e(sizes["scalar_len"], i32),
            "in_h": e(sizes["scalar_len"], i32), "out_x": e(sizes["scalar_len"], i32),
            "out_h": e(sizes["scalar_len"], i32), "llh_site": e(sizes["site_len"], f64),
            "root_lr": e(sizes["site_len"], f32), "root_x": e(sizes["site_len"], i32),
            "cnt_part": e(sizes["count_floats"], f32),
            "barrier": torch.zeros(2, dtype=i32, device=dev),
            "error": torch.zeros(1, dtype=i32, device=dev),
            # item / group descriptors, built on the device below
            "in_desc": e(12 * sizes["n_in_items"], i32),
            "out_desc": e(12 * sizes["n_out_items"], i32),
            "grp_desc": e(8 * sizes["n_groups_total"], i32),
        }
        if ultrametric:
            self.work["nd_uwork"] = e(N.UWORK_SLOTS * nn, f64)
        if want_post:
            self.work["post0"] = e(sizes["post_len"], f32)
            self.work["post1"] = e(sizes["post_len"], f32)
        self.b = N.Batch()
        b = self.b
        b.group_sites, b.compat, b.n_trees, b.n_datasets = G, int(compat), T, D
        b.n_nodes = nn
        b.n_in_levels, b.n_out_levels = sizes["n_in_levels"], sizes["n_out_levels"]
        b.n_in_items, b.n_out_items = sizes["n_in_items"], sizes["n_out_items"]
        b.n_root_items = sizes["n_root_items"]
        # the largest group: sizes the staged kernels' shared-memory row buffers
        b.max_states = int(max(int(np.max(x.group_C)) for x in datasets))
        # the largest tree: whether the M-step needs its cluster kernel
        b.max_tree_nodes = int(max(t.num_nodes for t in trees))
        b.plan_part_floats = int(sizes["part_floats"])
        b.plan_scalar_len = int(sizes["scalar_len"])
        for name, _ in N.BATCH_FIELDS:
            if name in v:
                setattr(b, name, v[name].data_ptr())
            elif name in self.work:
                setattr(b, name, self.work[name].data_ptr())
        if not want_post:
            b.post0 = None
            b.post1 = None
        # host copies of the level offsets: per-level launches need no read-back
        self._h_in_off = np.ascontiguousarray(plan["in_level_off"], np.int32)
        self._h_out_off = np.ascontiguousarray(plan["out_level_off"], np.int32)
        b.h_in_level_off = self._h_in_off.ctypes.data
        b.h_out_level_off = self._h_out_off.ctypes.data
        self._stream_ptr = (stream.cuda_stream if stream is not None
                            else torch.cuda.current_stream(self.device).cuda_stream)
        N.check(N.lib().laml_plan_descriptors(
            C.byref(b), b.in_desc, b.out_desc, b.grp_desc, self._s()))

    @property
    def lbfgs(self) -> bool:
        """fastEM model: run the M-step the reference itself runs (100 FP32
        L-BFGS steps, fast_em/laml.py:49-110) instead of solving its
        objective to the stationary point; allocates its vectors on first
        use."""
        return self._lbfgs

    @lbfgs.setter
    def lbfgs(self, on: bool):
        if on and not self.compat:
            raise ValueError("the L-BFGS M-step is the fastEM (compat) model's")
        if on and "nd_lbfgs" not in self.work:
            n = N.LBFGS_SLOTS * (self.sizes["n_nodes"] + 2 * self.T)
            self.work["nd_lbfgs"] = torch.zeros(n, dtype=torch.float32, device=self.device)
            self.b.nd_lbfgs = self.work["nd_lbfgs"].data_ptr()
        self._lbfgs = bool(on)

    @property
    def wide_chunk(self) -> int:
        """The wide levels' kernel: 0 per-thread row loads (default), 8 or 16
        bulk-staged rows with that many state slots per stage.  A tiling
        choice: the results are bitwise the same."""
        return int(self.b.wide_chunk)

    @wide_chunk.setter
    def wide_chunk(self, ch: int):
        if ch not in (0, 8, 16):
            raise ValueError("wide_chunk must be 0, 8 or 16")
        self.b.wide_chunk = int(ch)

    @property
    def wide_pc(self) -> bool:
        """Run the wide levels on producer/consumer warp pairs (a producer
        warp bulk-copies rows and per-site scalars into shared memory for its
        consumer warp; ``wide_chunk`` state slots per stage, 0 = 8).  A tiling
        choice: the results are bitwise the same."""
        return bool(self.b.wide_pc)

    @wide_pc.setter
    def wide_pc(self, on: bool):
        self.b.wide_pc = 1 if on else 0

    # -- raw entry points -------------------------------------------------
    def _s(self):
        return C.c_void_p(self._stream_ptr)

    def branch_terms(self):
        N.check(N.lib().laml_branch_terms(C.byref(self.b), self._s()))

    def inside(self, update_em=False):
        N.check(N.lib().laml_inside(C.byref(self.b), int(update_em), self._s()))

    def outside(self, want_post=False, true_root=False):
        flags = (N.OUT_POSTERIORS if want_post else 0) | (N.OUT_TRUE_ROOT if true_root else 0)
        N.check(N.lib().laml_outside(C.byref(self.b), flags, self._s()))

    def gradient(self):
        """(grad_d [n_nodes], grad_nu [T], grad_phi [T]) as float64 device
        tensors, from the counts of outside(true_root=True)."""
        gd = torch.empty(self.sizes["n_nodes"], dtype=torch.float64, device=self.device)
        gp = torch.empty(2 * self.T, dtype=torch.float64, device=self.device)
        N.check(N.lib().laml_gradient(C.byref(self.b), gd.data_ptr(), gp.data_ptr(), self._s()))
        return gd, gp[0::2], gp[1::2]

    def set_params(self, d=None, nu=None, phi=None):
        """Overwrite branch lengths (float64 [n_nodes]) / nu / phi ([T]) from
        device or host tensors."""
        if d is not None:
            self.v["nd_d"].copy_(torch.as_tensor(d, dtype=torch.float64).reshape(-1))
        if nu is not None:
            self.v["tr_nu"].copy_(torch.as_tensor(nu, dtype=torch.float64).reshape(-1))
        if phi is not None:
            self.v["tr_phi"].copy_(torch.as_tensor(phi, dtype=torch.float64).reshape(-1))

    def _polish(self, polish):
        # the exact (EM_solver) model polishes its solves in FP64 by default
        return (not self.compat) if polish is None else bool(polish)

    def _mflags(self, polish):
        return ((N.MSTEP_FP64_POLISH if self._polish(polish) else 0) |
                (N.MSTEP_ULTRAMETRIC if self.ultrametric else 0) |
                (N.MSTEP_ULTRA_BARRIER if self.ultra_barrier else 0) |
                (N.MSTEP_ULTRA_PD_SHORT if self.ultra_pd_short else 0) |
                (N.MSTEP_LBFGS if self._lbfgs else 0))

    def mstep(self, rounds=MSTEP_ROUNDS, polish=None):
        N.check(N.lib().laml_mstep(C.byref(self.b), rounds, self._mflags(polish), self._s()))

    def em_iterations(self, iters, rounds=MSTEP_ROUNDS, rel_tol=None, max_iters=100000,
                      persistent=True, polish=None):
        tol = rel_tol if rel_tol is not None else (EM_STOP_COMPAT if self.compat else EM_STOP_EXACT)
        f = N.lib().laml_em_run if persistent else N.lib().laml_em_run_levels
        N.check(f(C.byref(self.b), iters, rounds, tol, max_iters, self._mflags(polish),
                  self._s()))

    def em_graph(self, iters=1, rounds=MSTEP_ROUNDS, rel_tol=None, max_iters=100000,
                 persistent=False, polish=None):
        """A CUDA graph of ``iters`` EM iterations on this batch (replay with
        ``launch_graph``); cached per argument set."""
        tol = rel_tol if rel_tol is not None else (EM_STOP_COMPAT if self.compat else EM_STOP_EXACT)
        key = (iters, rounds, tol, max_iters, bool(persistent), self._mflags(polish),
               self.wide_chunk, self.wide_pc)
        if not hasattr(self, "_graphs"):
            self._graphs = {}
        if key not in self._graphs:
            h = C.c_void_p()
            N.check(N.lib().laml_em_graph_create(
                C.byref(self.b), iters, rounds, tol, max_iters, key[5], int(persistent),
                C.byref(h)))
            self._graphs[key] = h
        return self._graphs[key]

    def em_graph_loop(self, chunk=4, rounds=MSTEP_ROUNDS, rel_tol=None, max_iters=100000,
                      polish=None):
        """A CUDA graph that runs EM to convergence in one launch: a device-side
        WHILE loop over ``chunk``-iteration bodies that stops when no tree is
        ACTIVE (laml_em_graph_loop_create); cached per argument set."""
        tol = rel_tol if rel_tol is not None else (EM_STOP_COMPAT if self.compat else EM_STOP_EXACT)
        max_chunks = (max_iters + chunk - 1) // chunk + 1
        key = ("loop", chunk, rounds, tol, max_iters, self._mflags(polish), self.wide_chunk,
               self.wide_pc)
        if not hasattr(self, "_graphs"):
            self._graphs = {}
        if key not in self._graphs:
            h = C.c_void_p()
            # the graph's chunk counter: one device int per graph, zero between launches
            cnt = torch.zeros(1, dtype=torch.int32, device=self.device)
            self.work[f"loop_counter_{len(self._graphs)}"] = cnt
            N.check(N.lib().laml_em_graph_loop_create(
                C.byref(self.b), chunk, rounds, tol, max_iters, key[5], max_chunks,
                C.c_void_p(cnt.data_ptr()), C.byref(h)))
            self._graphs[key] = h
        return self._graphs[key]

    def launch_graph(self, g):
        N.check(N.lib().laml_graph_launch(g, self._s()))

    def __del__(self):
        for g in getattr(self, "_graphs", {}).values():
            try:
                N.lib().laml_graph_destroy(g)
            except Exception:
                pass

    def check_device_error(self):
        err = int(self.work["error"].item())
        if err != 0:
            raise N.LamlError(err, "device-side error (grid barrier timeout)")

    # -- composite operations --------------------------------------------
    def log_likelihood(self):
        """Per-tree log-likelihood (FP64) at the current parameters."""
        self.branch_terms()
        self.inside(update_em=False)
        return self.work["tr_llh"].cpu().numpy().copy()

    def e_step(self, want_post=False):
        """Inside + outside + counts at the current parameters."""
        self.branch_terms()
        self.inside(update_em=True)
        self.outside(want_post=want_post)
        self.counts_from_partials()

    def counts_from_partials(self):
        """Sum the per-group count partials into nd_cnt (6 per node) without
        an M-step: the raw E-step counts of calc.compute_E_step."""
        cp = self.work["cnt_part"]
        out = np.zeros((self.sizes["n_nodes"], 6))
        lr = []
        cnt = cp.cpu().numpy()
        base = self.v["tr_cnt_base"].cpu().numpy()
        nb = self.v["tr_node_base"].cpu().numpy()
        for p, t in enumerate(self.trees):
            ng = self.datasets[self.tree_ds[p]].n_groups
            blk = cnt[base[p]:base[p] + t.num_nodes * ng * 8].reshape(t.num_nodes, ng, 8)
            s = blk.astype(np.float64).sum(axis=1)
            out[nb[p]:nb[p] + t.num_nodes] = s[:, :6]
            lr.append(s[:, 6] + s[:, 7])
        self._counts = out
        self._leaf_resp = lr
        return out, lr

    def run_em(self, rounds=MSTEP_ROUNDS, rel_tol=None, max_iters=100000, chunk=4,
               persistent=None, polish=None, path=None):
        """EM to convergence for every tree: inside at the start parameters,
        then chunks of ``chunk`` fused iterations until no tree is ACTIVE.
        ``path``: "graph" (one launch of a CUDA graph whose device-side WHILE
        node repeats ``chunk`` iterations of per-level launches until no tree
        is ACTIVE; the default), "levels" (the same launches issued directly,
        the host testing convergence after every chunk) or "persistent" (one
        cooperative kernel per chunk); ``persistent`` True / False is
        shorthand for "persistent" / "levels"."""
        if path is None:
            path = "graph" if persistent is None else ("persistent" if persistent else "levels")
        if path not in ("graph", "levels", "persistent"):
            raise ValueError(f"unknown EM path {path!r}")
        if path == "graph":
            self.run_em_start(rounds=rounds, rel_tol=rel_tol, max_iters=max_iters, chunk=chunk,
                              polish=polish)
            return self.run_em_finish()
        self.branch_terms()
        self.inside(update_em=True)
        done = 0
        while True:
            self.em_iterations(chunk, rounds=rounds, rel_tol=rel_tol, max_iters=max_iters,
                               persistent=path == "persistent", polish=polish)
            done += chunk
            st = self.work["tr_status"]
            if not bool((st == N.TREE_ACTIVE).any()):
                break
            if done >= max_iters + chunk:
                break
        if path == "persistent":
            self.check_device_error()
        return self.results()

    def run_em_start(self, rounds=MSTEP_ROUNDS, rel_tol=None, max_iters=100000, chunk=4,
                     polish=None):
        """Queue EM to convergence on the batch's stream without waiting: the
        start-parameter inside pass, then one launch of the EM loop graph (the
        whole loop runs on the device; its chunk cap is past every tree's
        iteration cap).  ``run_em_finish`` waits and returns the results."""
        self.branch_terms()
        self.inside(update_em=True)
        g = self.em_graph_loop(chunk, rounds=rounds, rel_tol=rel_tol, max_iters=max_iters,
                               polish=polish)
        self.launch_graph(g)

    def run_em_finish(self) -> List[TreeResult]:
        """Wait for ``run_em_start``'s work and return the per-tree results."""
        self.check_device_error()
        return self.results()

    def results(self) -> List[TreeResult]:
        """Per-tree results, fetched with one device->host copy."""
        T, nn = self.T, self.sizes["n_nodes"]
        w, v = self.work, self.v
        dev = torch.cat([w["tr_llh"].view(-1), v["tr_nu"].view(-1), v["tr_phi"].view(-1),
                         w["tr_prev"].view(-1), v["nd_d"].view(-1), w["nd_d_prev"].view(-1),
                         w["tr_iter"].to(torch.float64), w["tr_status"].to(torch.float64)])
        nbytes = dev.numel() * 8
        stage = getattr(self, "_pinned", None)
        if stage is not None and stage.is_pinned() and stage.numel() >= nbytes:
            # the upload's pinned staging buffer (idle since the upload) takes
            # the copy: a DMA into page-locked memory, no fresh pageable
            # allocation to fault in; every tree's lengths are copied out of it
            hv = stage[:nbytes].view(torch.float64)
            hv.copy_(dev, non_blocking=True)
            torch.cuda.current_stream(self.device).synchronize()
            host = hv.numpy()
        else:
            host = dev.cpu().numpy()
        self.last_d2h_bytes = host.nbytes
        o = 0
        llh = host[o:o + T]; o += T
        nu = host[o:o + T]; o += T
        phi = host[o:o + T]; o += T
        prev = host[o:o + 2 * T].reshape(-1, 2); o += 2 * T
        d = host[o:o + nn]; o += nn
        dprev = host[o:o + nn]; o += nn
        it = host[o:o + T].astype(np.int64); o += T
        st = host[o:o + T].astype(np.int64)
        nb = self._node_base
        out = []
        for p, t in enumerate(self.trees):
            sl = slice(nb[p], nb[p] + t.num_nodes)
            old = self.compat and st[p] in (N.TREE_CONVERGED, N.TREE_NAN) and it[p] > 0
            if st[p] == N.TREE_NAN and not self.compat:
                old = True
            if old:
                # fast_em/laml.py:183-194 returns the parameters before the
                # last M-step (the loop breaks before params = new_params)
                out.append(TreeResult(float(llh[p]), float(prev[p, 0]), float(prev[p, 1]),
                                      int(it[p]), int(st[p]), dprev[sl].copy()))
            else:
                out.append(TreeResult(float(llh[p]), float(nu[p]), float(phi[p]), int(it[p]),
                                      int(st[p]), d[sl].copy()))
        return out

    # -- per-site / per-node views ---------------------------------------
    def site_llh(self, p):
        """Per original site log-likelihood of tree p."""
        ds = self.datasets[self.tree_ds[p]]
        base = int(self.v["tr_site_base"][p].item())
        v = self.work["llh_site"][base:base + ds.n_sites_pad].cpu().numpy()
        out = np.empty(ds.n_sites)
        for c in range(ds.n_sites_pad):
            o = ds.site_perm[c]
            if o >= 0:
                out[o] = v[c]
        return out

    def posteriors(self, p):
        """(P(v=0|D), P(v=silenced|D)) as float arrays [N, K] in original site
        order (needs want_post=True and outside(want_post=True))."""
        ds = self.datasets[self.tree_ds[p]]
        t = self.trees[p]
        base = int(self.v["tr_post_base"][p].item())
        n = t.num_nodes * ds.n_sites_pad
        a0 = self.work["post0"][base:base + n].cpu().numpy().reshape(t.num_nodes, ds.n_sites_pad)
        a1 = self.work["post1"][base:base + n].cpu().numpy().reshape(t.num_nodes, ds.n_sites_pad)
        keep = ds.site_perm >= 0
        o0 = np.empty((t.num_nodes, ds.n_sites), np.float32)
        o1 = np.empty_like(o0)
        o0[:, ds.site_perm[keep]] = a0[:, keep]
        o1[:, ds.site_perm[keep]] = a1[:, keep]
        return o0, o1

    @property
    def h2d_bytes(self):
        return self._h2d_bytes


class _nullctx:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False
