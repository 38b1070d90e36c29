"""Benchmark: batched PMM EM on 512 NNI candidates of a 1000-leaf Yule tree.

Workload (seeded synthetic data, the shapes of the batched NNI-scoring
configuration): one 1,000-leaf Yule tree (branch lengths ~ Exp(mean 0.1),
floor 0.006) and 511 random NNI neighbours; a shared 40-site matrix simulated
under PMM (nu = 0.1, phi = 0.15, M_k ~ U{5..50}, q ~ Dirichlet(0.5)); fastEM
(compat) semantics.

A step is one EM iteration over the whole batch (outside + expected counts ->
M-step -> inside + log-likelihood): one replay of a CUDA graph of the
per-level launches (``--path``).  ``value`` is tree-EM-iterations per second
with the batch resident in HBM (convergence disabled so every step does the
full work; the partial buffers, ~2.6 GB, are far larger than L2, so no flush
is needed).  ``roofline`` is the outside pass (the dominant kernel), timed
alone on the same stream; ``roofline_inside`` and ``roofline_em_iteration``
give the inside pass and the whole iteration.  ``e2e`` scores the same 512
candidates through the public API (api.score_candidates) from host newick
strings and the host character matrix to converged results back on the host,
timed by wall clock with the copies inside; ``plain_gpu_dropin`` scores a
sample of candidates one at a time through the drop-in solver, the way the
reference's topology search calls it.

--impl reference times the CPU restatement of the reference's fastEM path
(the oracle port) on the host cores, on a bounded sample of the same
workload.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "EM iters/s & node-site updates/s, batched+served vs plain GPU; p50/p99 latency"
# DRAM bytes per launch of the outside and inside passes of the 512-candidate
# batch (G = 8, per-thread wide kernels): ncu dram__bytes_read.sum +
# dram__bytes_write.sum summed over one pass of the first 128 candidates
# (`--passes-only --trees 128 --wide-chunk 0`), times 4 -- the full batch holds
# 4x the same-shaped rows -- over the pass's launches (outside 25, inside 24)
TRAFFIC_PER_LAUNCH = {"outside": 175.9e6, "inside": 119.6e6}
UNIT = "tree-EM-iters/s"
WORKLOAD = "nni512"


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def pass_bytes(b):
    """Algorithmic bytes of one inside pass, one outside pass and one M-step
    in this layout (A = 4 B x part_floats, one FP32 partial array over the
    internal nodes):

    * inside: every internal row written once and read once by its parent
      (2A); per internal (node, site) 12 B of scalars (exponent, cumulative
      exponent, q-dot) written and read (24 B); leaf codes 2 B per leaf site;
      16 B of branch terms per node.
    * outside, one item per internal parent for both children: the parent's
      outside row, the children's inside rows and the children's outside rows
      once each (3A); scalars 8 B read + 12 B read + 8 B written per internal
      (node, site); leaf codes; branch terms; count partials written (32 B
      per (node, group)).
    * M-step: count partials read, branch lengths read and written, branch
      terms written (16 + 16 B per node)."""
    leaf_sites = sum(t.num_leaves * b.datasets[b.tree_ds[p]].n_sites_pad
                     for p, t in enumerate(b.trees))
    return _pass_bytes(b.sizes, leaf_sites)


def request_bytes(tree, ds):
    """pass_bytes of a one-tree batch of a request, from the host plan."""
    from laml_gb300.encoding import plan_batch
    sizes, _ = plan_batch([tree], [0], [ds], host_desc=False)
    return _pass_bytes(sizes, tree.num_leaves * ds.n_sites_pad)


def _pass_bytes(s, leaf_sites):
    A = 4 * s["part_floats"]
    nn = s["n_nodes"]
    inside = 2 * A + 24 * s["scalar_len"] + 2 * leaf_sites + 16 * nn
    outside = 3 * A + 28 * s["scalar_len"] + 2 * leaf_sites + 16 * nn + 4 * s["count_floats"]
    mstep = 4 * s["count_floats"] + 32 * nn
    return {"inside": inside, "outside": outside, "mstep": mstep,
            "em_iteration": inside + outside + mstep}


def plain_dropin(w, n, device):
    """The plain drop-in: candidates one at a time through the fastEM_solver
    mirror (one solver object, one EM to convergence per candidate), as the
    reference's topology search calls its solver."""
    import torch

    from laml_gb300.fastEM_solver import fastEM_solver
    data = {"charMtrx": w.rows, "ordered_leaf_labels": [w.leaf_order]}
    prior = {"Q": w.Q}
    fastEM_solver([w.newicks[0]], data, prior, device=device).score_tree()   # warm
    torch.cuda.synchronize(device)
    iters, t0 = 0, time.perf_counter()
    for nw in w.newicks[:n]:
        s = fastEM_solver([nw], data, prior, device=device)
        s.score_tree()
        iters += s.last_em_iterations
    return iters / (time.perf_counter() - t0)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_sample_port(workload, n_trees, iters):
    """Oracle port (FP64, log space) on `n_trees` candidates x `iters` EM
    iterations, one process per core; returns (tree-EM-iters/s, cores)."""
    from oracle import cpu_port
    return cpu_port.em_throughput(workload, n_trees, iters)


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return
    from laml_gb300 import synth
    w = synth.workload_config(WORKLOAD, seed=args.seed)
    per_step = args.ref_trees
    vals = []
    cores = None
    for i in range(args.warmup + args.steps):
        v, cores = cpu_sample_port(w, per_step, 1)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step / value * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": "512 NNI candidates of a 1000-leaf Yule tree, 40 sites, "
                                   "M~U{5..50}, fastEM semantics", "sample_trees": per_step},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{per_step} of the 512 candidates x 1 EM iteration per "
                                       f"step, FP64 C restatement, one tree per core"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_serving(args, emit=True):
    """Poisson stream of PMM requests (leaves log-uniform 200-10,000, sites
    U(30, 300), M_k ~ U{5..100}, nu ~ U(0, 0.2), phi ~ U(0, 0.3), Yule trees)
    through the continuous-batching server; half log-likelihood requests,
    half EM-to-convergence requests.  A pool of seeded problems is drawn once
    (generation is not timed); arrivals are replayed in real time."""
    import numpy as np
    import torch

    import concurrent.futures as cf

    from laml_gb300 import serving as S
    from laml_gb300 import synth

    rng = np.random.default_rng(args.seed + 7)
    pool = []
    for i in range(args.serve_pool):
        n = int(round(math.exp(rng.uniform(math.log(200), math.log(10000)))))
        K = int(rng.integers(30, 301))
        nu, phi = float(rng.uniform(0, 0.2)), float(rng.uniform(0, 0.3))
        w = synth.pmm_workload(n, K, 5, 100, 0.5, nu, phi, seed=args.seed + 1000 + i)
        pool.append(w)
    rate, dur = args.serve_rate, args.serve_seconds
    t, arrivals = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > dur:
            break
        arrivals.append((t, int(rng.integers(len(pool))), "llh" if rng.random() < 0.5 else "em"))
    srv = S.PMMServer(hbm_budget=args.serve_budget << 30, graphs=not args.serve_no_graphs,
                      chunk=args.serve_chunk, max_em_cohort=args.serve_em_cohort)
    # each client's matrix is encoded once (as a search client scoring many
    # trees against it would), outside the timed replay
    dsets = [srv.encode_dataset(w.rows, w.Q, w.leaf_order) for w in pool]
    # algorithmic bytes of one inside pass and one EM iteration per problem,
    # for the capacity arithmetic of the line
    from laml_gb300.encoding import encode_newick
    pbytes = [request_bytes(encode_newick(w.newicks[0], w.leaf_order), ds)
              for w, ds in zip(pool, dsets)]
    # warm the kernels and the allocator with one small request of each kind
    for kind in ("llh", "em"):
        w = pool[0]
        srv.submit(S.Request(w.newicks[0], w.rows, w.Q, w.leaf_order, kind=kind,
                             dataset=dsets[0])).result()
    futs = []
    t0 = time.perf_counter()
    with Clocks(0) as clk:
        for (ta, k, kind) in arrivals:
            now = time.perf_counter() - t0
            if ta > now:
                time.sleep(ta - now)
            w = pool[k]
            futs.append((kind, k, srv.submit(S.Request(w.newicks[0], w.rows, w.Q, w.leaf_order,
                                                       kind=kind, dataset=dsets[k]))))
        # wait for the replies up to a drain deadline after the last arrival;
        # the offered EM load can exceed what one GPU completes (each EM
        # request is tens of iterations over up to 10,000 leaves x 300
        # sites), so requests still running then are reported, not awaited
        deadline = time.perf_counter() + args.serve_drain
        replies, unfinished = [], {"llh": 0, "em": 0}
        for kind, k, f in futs:
            try:
                replies.append((kind, f.result(timeout=max(0.0, deadline - time.perf_counter())), k))
            except cf.TimeoutError:
                unfinished[kind] += 1
        t_end = time.perf_counter()
        stuck = srv.snapshot() if any(unfinished.values()) else []
        launched = srv.em_tree_iterations
        completed_iters = srv.em_tree_iterations_completed
        recohorts = srv.recohorts
    srv.close(wait=not any(unfinished.values()))
    lat = np.array([r.latency for _, r, _ in replies]) if replies else np.zeros(1)
    lat_em = np.array([r.latency for k, r, _ in replies if k == "em"])
    lat_llh = np.array([r.latency for k, r, _ in replies if k == "llh"])
    iters = sum(r.result.iterations for _, r, _ in replies)
    span = t_end - t0
    # capacity: algorithmic bytes of the answered requests (an EM request:
    # its iterations x one EM iteration; a likelihood request: one inside
    # pass), over the stream's length (offered) and over the time to the
    # last answer (sustained)
    em_req_b = [r.result.iterations * pbytes[k]["em_iteration"]
                for kind, r, k in replies if kind == "em"]
    llh_b = sum(pbytes[k]["inside"] for kind, _, k in replies if kind == "llh")
    work_b = float(sum(em_req_b) + llh_b)
    # value: tree-EM-iterations of the requests answered by the end of the
    # window, per second of the window (useful work; launched iterations of
    # requests still running are reported apart)
    n_em = sum(1 for _, _, k in arrivals if k == "em")
    line = {"metric": METRIC, "mode": "serving", "value": completed_iters / span, "unit": UNIT,
            "em_iterations_of_completed_requests": iters,
            "em_tree_iterations_launched_per_s": launched / span,
            "em_requests": n_em, "em_completed_fraction":
                (n_em - unfinished["em"]) / n_em if n_em else None,
            "recohorts": recohorts,
            "unfinished_em_on_device": stuck[:12],
            "n_gpus": 1, "requests": len(futs), "completed": len(replies),
            "unfinished_at_deadline": unfinished, "drain_deadline_s": args.serve_drain,
            "offered_rate_per_s": rate, "completed_per_s": len(replies) / span,
            "capacity": {
                "algorithmic_gb": work_b / 1e9,
                "offered_gb_per_s": work_b / dur / 1e9,
                "sustained_gb_per_s": work_b / span / 1e9,
                "em_request_gb_median": float(np.median(em_req_b)) / 1e9 if em_req_b else None,
                "em_request_gb_max": float(max(em_req_b)) / 1e9 if em_req_b else None,
                "basis": "answered requests only; bench.pass_bytes per request plan"},
            "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)),
            "p50_latency_em_s": float(np.percentile(lat_em, 50)) if len(lat_em) else None,
            "p99_latency_em_s": float(np.percentile(lat_em, 99)) if len(lat_em) else None,
            "p50_latency_llh_s": float(np.percentile(lat_llh, 50)) if len(lat_llh) else None,
            "p99_latency_llh_s": float(np.percentile(lat_llh, 99)) if len(lat_llh) else None,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "Poisson requests, leaves log-U(200,10000), sites U(30,300), "
                                   "M_k U{5..100}, nu U(0,0.2), phi U(0,0.3); half llh, half EM",
                       "pool": len(pool), "seconds": dur, "hbm_budget_gb": args.serve_budget,
                       "chunk": args.serve_chunk, "max_em_cohort": args.serve_em_cohort,
                       "graphs": not args.serve_no_graphs},
            "clocks": clk.summary()}
    if emit:
        print(json.dumps(line), flush=True)
    return line


def run_passes_only(args):
    """One inside and one outside pass of the first --trees candidates, no
    timing: the command the kernel profiles are captured on."""
    import torch

    from laml_gb300 import problem as PB
    from laml_gb300 import synth
    w = synth.workload_config(WORKLOAD, seed=args.seed)
    w.newicks = w.newicks[:args.trees]
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True,
                      group_sites=args.group_sites or 8, nu=0.5, phi=0.5)
    b.wide_chunk = max(args.wide_chunk, 0)
    b.wide_pc = args.wide_pc > 0
    b.branch_terms()
    b.inside(update_em=True)
    b.outside()
    torch.cuda.synchronize()
    b.check_device_error()
    print(json.dumps({"passes_only": True, "trees": b.T, "n_in_levels": b.sizes["n_in_levels"],
                      "n_out_levels": b.sizes["n_out_levels"]}), flush=True)


def _timed(fn, stream, reps):
    import torch
    fn()
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    stream.synchronize()
    return e0.elapsed_time(e1) / reps


def run_workload(args):
    """The other configurations, one JSON line each (rank 0, one GPU):

    * fixed250: one 250-leaf Yule tree, 30 sites, M_k ~ U{5..30}: negative_llh
      (one inside pass) and 50 EM iterations; the C restatement timed beside.
    * grad4096: one 4096-leaf tree, 100 sites, M_k ~ U{10..100}, q ~ Dir(0.3),
      nu = 0.05, phi = 0.1: forward log-likelihood plus the adjoint gradient
      in d (8,190 branches), nu, phi through torch.autograd.
    * large50k: one 50,000-leaf tree, 300 sites, M_k ~ U{20..100},
      q ~ Dir(0.2), nu = 0.1, phi = 0.2: EM until the relative log-likelihood
      change is below 1e-8, with the inside and outside passes timed alone
      for their HBM rooflines."""
    import numpy as np
    import torch

    from laml_gb300 import autograd as AG
    from laml_gb300 import problem as PB
    from laml_gb300 import synth

    name = args.workload
    w = synth.workload_config(name, seed=args.seed)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)
    peak, peak_kind = peaks()
    nu0, phi0 = {"fixed250": (0.1, 0.15), "grad4096": (0.05, 0.1), "large50k": (0.1, 0.2)}[name]
    with torch.cuda.stream(stream):
        b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, group_sites=8,
                          nu=nu0, phi=phi0, device=dev, stream=stream)
    ds = b.datasets[0]
    cfg = {"workload": name, "leaves": b.trees[0].num_leaves, "sites": ds.n_sites,
           "nodes": b.sizes["n_nodes"], "group_sites": 8,
           "partial_buffer_gb": 4 * b.sizes["part_floats"] / 1e9}
    line = {"metric": METRIC, "mode": name, "n_gpus": 1, "dtype": "f32", "data": "synthetic",
            "config": cfg}
    pb = pass_bytes(b)
    with torch.cuda.stream(stream):
        b.branch_terms()
        ms_in = _timed(lambda: b.inside(update_em=True), stream, max(3, args.steps))
        ms_out = _timed(lambda: b.outside(), stream, max(3, args.steps))
    line["inside_ms"], line["outside_ms"] = ms_in, ms_out
    line["roofline_inside"] = {"bound": "hbm", "achieved": pb["inside"] / ms_in / 1e6,
                               "peak": peak, "unit": "GB/s",
                               "frac": pb["inside"] / ms_in / 1e6 / peak, "peak_kind": peak_kind}
    line["roofline"] = {"bound": "hbm", "achieved": pb["outside"] / ms_out / 1e6, "peak": peak,
                        "unit": "GB/s", "frac": pb["outside"] / ms_out / 1e6 / peak,
                        "peak_kind": peak_kind, "kernel": "outside pass (all levels)"}
    if name == "fixed250":
        with torch.cuda.stream(stream):
            ms_llh = _timed(lambda: b.inside(update_em=False), stream, 20)
            iters = 50

            graph = b.em_graph(iters, rel_tol=-1.0, max_iters=1 << 30, persistent=False)

            def em50():   # the solver's path: one CUDA-graph replay of 50 iterations
                b.set_params(d=np.maximum(b.trees[0].branch_length, 1e-6), nu=[nu0], phi=[phi0])
                b.branch_terms()
                b.inside(update_em=True)
                b.launch_graph(graph)
            ms_em = _timed(em50, stream, max(3, args.steps))
        line.update({"value": iters / (ms_em / 1e3), "unit": "EM iters/s",
                     "negative_llh_ms": ms_llh, "em50_ms": ms_em,
                     "negative_llh": -float(b.work["tr_llh"][0].item())})
        if not args.no_cpu:
            from oracle import cpu_port
            t0 = time.perf_counter()
            cpu_port.em(w.newicks, w.rows, w.Q, w.leaf_order, nu0, phi0, iters=iters)
            dt = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": iters / dt, "unit": "EM iters/s", "cores": 1,
                                    "kind": "port", "sample": "the same tree, 50 EM "
                                    "iterations, FP64 C restatement, one core"}
    elif name == "grad4096":
        d = b.v["nd_d"].clone().requires_grad_(True)
        nu = b.v["tr_nu"].clone().requires_grad_(True)
        phi = b.v["tr_phi"].clone().requires_grad_(True)

        def fb():
            for t in (d, nu, phi):
                t.grad = None
            AG.log_likelihood(d, nu, phi, b).sum().backward()
        with torch.cuda.stream(stream):
            ms_fb = _timed(fb, stream, max(3, args.steps))
            ms_f = _timed(lambda: AG.log_likelihood(d, nu, phi, b), stream, max(3, args.steps))
        line.update({"value": 1e3 / ms_fb, "unit": "forward+adjoint evaluations/s",
                     "forward_ms": ms_f, "forward_backward_ms": ms_fb,
                     "grad_norm_d": float(d.grad.norm().item()),
                     "grad_nu": float(nu.grad[0].item()), "grad_phi": float(phi.grad[0].item())})
    else:   # large50k: EM to convergence
        with torch.cuda.stream(stream):
            # untimed warm-up: the EM graph run_em replays (instantiated and
            # cached here) and a first launch of the M-step and likelihood
            # kernels; the parameters are restored before the timed run
            b.em_graph(8, rel_tol=1e-8, max_iters=2000, persistent=False)
            d0 = b.v["nd_d"].clone()
            b.log_likelihood()
            b.mstep()
            b.set_params(d=d0, nu=[nu0], phi=[phi0])
            stream.synchronize()
            t0 = time.perf_counter()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res = b.run_em(rel_tol=1e-8, max_iters=2000, chunk=8)
            e1.record(stream)
            stream.synchronize()
            wall = time.perf_counter() - t0
        r = res[0]
        ms = e0.elapsed_time(e1)
        line.update({"value": r.iterations / (ms / 1e3), "unit": "EM iters/s",
                     "em_iterations": r.iterations, "em_seconds": ms / 1e3,
                     "wall_seconds": wall, "llh": r.llh, "status": r.status,
                     "node_site_updates_per_s": 2.0 * b.sizes["n_nodes"] * ds.n_sites *
                     r.iterations / (ms / 1e3)})
    b.check_device_error()
    print(json.dumps(line), flush=True)


def run_ultra(args):
    """ultra250: EM_solver's default final optimisation (runner.py:287 calls
    optimize with ultra_constr=True) on the 250-leaf, 30-site configuration:
    the exact EM from a random start (ML_solver.ini_all's ranges) with every
    M-step solved under the ultrametric equalities, to the 1e-8 stopping
    rule.  One JSON line: EM iterations/s over the whole run, the time of
    one ultrametric M-step alone, and the oracle's ultrametric EM (NumPy E-step,
    LP start + dense barrier M-step) timed on the same tree for 3 iterations."""
    import numpy as np
    import torch

    from laml_gb300 import problem as PB
    from laml_gb300 import synth

    w = synth.workload_config("fixed250", seed=args.seed)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)
    rng = np.random.default_rng(args.seed + 7)
    trees = PB.encode_trees(w.newicks, w.leaf_order)
    N_ = trees[0].num_nodes
    d0 = rng.uniform(2 * 0.005, 10.0 / 2, N_)        # ML_solver.ini_all's range
    nu0, phi0 = float(rng.random() * 0.99), float(rng.random() * 0.99)
    if args.mstep_only:   # one E-step and one ultrametric M-step: the profiled command
        b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=False, nu=nu0,
                          phi=phi0, d=[d0], clamp=False, ultrametric=True, device=dev,
                          trees=trees)
        b.e_step()
        b.mstep()
        torch.cuda.synchronize()
        b.check_device_error()
        print(json.dumps({"mstep_only": True, "nodes": N_}), flush=True)
        return
    with torch.cuda.stream(stream):
        b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=False, nu=nu0, phi=phi0,
                          d=[d0], clamp=False, ultrametric=True, device=dev, stream=stream,
                          trees=trees)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        r = b.run_em(max_iters=1000, chunk=4)[0]
        e1.record(stream)
        stream.synchronize()
        wall = time.perf_counter() - t0
        ms = e0.elapsed_time(e1)
        b.e_step()
        ms_m = _timed(lambda: b.mstep(), stream, max(3, min(args.steps, 10)))
    b.check_device_error()
    t = trees[0]
    paths = []
    for leaf in range(t.num_leaves):
        x, acc = leaf, 0.0
        while t.parent[x] >= 0:
            acc += r.branch_lengths[x]
            x = t.parent[x]
        paths.append(acc)
    ds = b.datasets[0]
    line = {"metric": METRIC, "mode": "ultra250", "n_gpus": 1, "dtype": "f64 heights, f32 cores",
            "data": "synthetic",
            "config": {"workload": "ultra250", "leaves": t.num_leaves, "sites": ds.n_sites,
                       "nodes": N_, "model": "exact (EM_solver)", "ultra_constr": True},
            "value": r.iterations / (ms / 1e3), "unit": "EM iters/s",
            "em_iterations": r.iterations, "em_seconds": ms / 1e3, "wall_seconds": wall,
            "ultrametric_mstep_ms": ms_m, "llh": r.llh, "status": r.status,
            "root_to_leaf_spread": float(np.ptp(paths))}
    if not args.no_cpu:
        from oracle import pmm_oracle as O
        tr = O.parse_tree(w.newicks[0], w.leaf_order)
        enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, compat=False)
        prob = O.Problem(tr, enc, False)
        t0 = time.perf_counter()
        O.em_exact(prob, d0, nu0, phi0, max_iters=3, stop=-1.0, ultra=True)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": 3 / dt, "unit": "EM iters/s", "cores": 1, "kind": "port",
                                "sample": "the same tree and start, 3 EM iterations of the "
                                          "oracle's ultrametric EM (NumPy FP64)"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--group-sites", type=int, default=0,
                    help="sites per group (0: the autotuner's choice)")
    ap.add_argument("--wide-chunk", type=int, default=-1,
                    help="wide levels: 0 per-thread loads, 8/16 bulk-staged rows with that many "
                         "slots per stage (-1: the autotuner's choice)")
    ap.add_argument("--wide-pc", type=int, default=-1,
                    help="wide levels on producer/consumer warp pairs: 1 on, 0 off "
                         "(-1: the autotuner's choice)")
    ap.add_argument("--no-other-paths", action="store_true",
                    help="skip timing the other EM-iteration drivers after the timed region")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--ref-trees", type=int, default=16)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--plain-trees", type=int, default=8,
                    help="candidates timed one at a time through the drop-in solver")
    ap.add_argument("--path", default="graph", choices=["graph", "persistent", "levels"],
                    help="graph: a CUDA graph of the per-level launches of one EM iteration "
                         "(one graph launch per step); persistent: one cooperative launch "
                         "per step; levels: the per-level launches issued directly")
    ap.add_argument("--trees", type=int, default=512,
                    help="use the first N candidates (smaller cases for profiling)")
    ap.add_argument("--workload", default="nni512",
                    choices=["nni512", "fixed250", "grad4096", "large50k", "ultra250"],
                    help="nni512 (the default bench line) or one of the other configurations")
    ap.add_argument("--mstep-only", action="store_true",
                    help="with --workload ultra250: one E-step and one ultrametric M-step "
                         "(profiling)")
    ap.add_argument("--passes-only", action="store_true",
                    help="one inside and one outside pass of --trees candidates (profiling)")
    ap.add_argument("--serving", action="store_true",
                    help="Poisson request stream through the continuous-batching server")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-seconds", type=float, default=5.0)
    ap.add_argument("--serve-pool", type=int, default=16)
    ap.add_argument("--serve-budget", type=int, default=64, help="HBM budget in GiB")
    ap.add_argument("--serve-chunk", type=int, default=4,
                    help="serving: EM iterations between cohort rebuilds")
    ap.add_argument("--serve-em-cohort", type=int, default=128,
                    help="serving: most EM requests in one cohort")
    ap.add_argument("--serve-no-graphs", action="store_true",
                    help="serving: EM chunks as per-level launches instead of graph replays")
    ap.add_argument("--no-serving", action="store_true",
                    help="leave the short serving stream out of the default line")
    ap.add_argument("--bench-serve-seconds", type=float, default=2.0,
                    help="seconds of Poisson arrivals of the default line's serving stream")
    ap.add_argument("--serve-drain", type=float, default=60.0,
                    help="seconds to wait for replies after the last arrival")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.serving:
        return run_serving(args)
    if args.workload == "ultra250":
        return run_ultra(args)
    if args.workload != "nni512":
        return run_workload(args)
    if args.passes_only:
        return run_passes_only(args)

    import numpy as np
    import torch
    import torch.distributed as dist

    from laml_gb300 import problem as PB
    from laml_gb300 import synth
    from laml_gb300 import tune
    from laml_gb300.api import score_candidates

    rank, world, local = _dist()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = synth.workload_config(WORKLOAD, seed=args.seed + rank)
    w.newicks = w.newicks[:args.trees]
    # the tile shape: sites per group x state slots per stage, timed on a
    # sample of the batch by the autotuner (not part of the timed region)
    tuned = None
    if args.group_sites and args.wide_chunk >= 0 and args.wide_pc >= 0:
        G, CH, PC = args.group_sites, args.wide_chunk, args.wide_pc > 0
    else:
        tuned = tune.autotune(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, device=dev)
        G = args.group_sites or tuned["group_sites"]
        CH = args.wide_chunk if args.wide_chunk >= 0 else tuned["wide_chunk"]
        PC = args.wide_pc > 0 if args.wide_pc >= 0 else bool(tuned.get("wide_pc", False))
    stream = torch.cuda.Stream(dev)
    with torch.cuda.stream(stream):
        b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, group_sites=G,
                          nu=0.5, phi=0.5, device=dev, stream=stream)
        b.wide_chunk = CH
        b.wide_pc = PC
        b.branch_terms()
        b.inside(update_em=True)
    stream.synchronize()   # the read below runs on the default stream
    llh_start = b.work["tr_llh"].cpu().numpy().copy()
    T = b.T
    nodes = b.sizes["n_nodes"]
    K = b.datasets[0].n_sites

    if args.path == "graph":
        with torch.cuda.stream(stream):
            graph = b.em_graph(1, rel_tol=-1.0, max_iters=1 << 30, persistent=False)

        def step():
            b.launch_graph(graph)
    else:
        def step():
            b.em_iterations(1, rel_tol=-1.0, max_iters=1 << 30,
                            persistent=args.path == "persistent")

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    if world > 1:
        dist.barrier()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with Clocks(local) as clk:
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        ev[0].record(stream)
        for i in range(args.steps):
            step()
            ev[i + 1].record(stream)
        stream.synchronize()
        t1 = time.perf_counter()
    b.check_device_error()

    # device time of the inside and the outside pass alone (their level
    # kernels), for the per-kernel roofline
    def pass_ms(fn, reps=5):
        fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / reps

    with torch.cuda.stream(stream):
        ms_out = pass_ms(lambda: b.outside())
        ms_in = pass_ms(lambda: b.inside(update_em=True))
    launch_ms = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[-1])
    if world > 1:
        tt = torch.tensor([total_ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
    ms = total_ms / args.steps
    value = T * world * args.steps / (total_ms / 1e3)
    nsu = 2.0 * nodes * K * world * args.steps / (total_ms / 1e3)
    pb = pass_bytes(b)
    avg_launch_s = statistics.mean(launch_ms) / 1e3
    peak, peak_kind = peaks()

    def roof(nbytes, seconds, kernel, launches):
        a = nbytes / seconds / 1e9
        return {"bound": "hbm", "achieved": a, "peak": peak, "unit": "GB/s", "frac": a / peak,
                "traffic": None, "kernel": kernel, "bytes_per_launch": nbytes / launches,
                "launches": launches, "seconds": seconds, "peak_kind": peak_kind}

    n_out, n_in = b.sizes["n_out_levels"], b.sizes["n_in_levels"]
    roof_out = roof(pb["outside"], ms_out / 1e3, "k_items outside levels (one launch per level "
                    "of internal parents, both children per item)", n_out + 2)
    roof_in = roof(pb["inside"], ms_in / 1e3, "k_items inside levels (one launch per height)",
                   n_in + 1)
    if T == 512 and G == 8 and CH == 0 and not PC:
        roof_out["traffic"] = TRAFFIC_PER_LAUNCH["outside"]
        roof_in["traffic"] = TRAFFIC_PER_LAUNCH["inside"]
    roof_it = roof(pb["em_iteration"], avg_launch_s,
                   {"graph": "EM-iteration graph (k_items per level, k_mstep)",
                    "persistent": "k_em_persistent",
                    "levels": "k_items per level, k_mstep"}[args.path], 1)
    llh_now = b.work["tr_llh"].cpu().numpy()
    with torch.cuda.stream(stream):
        # the other EM-iteration drivers on the same batch (after the timed
        # region): one cooperative persistent launch, or the per-level
        # launches without the graph
        ms_paths = {}
        for p_ in (() if args.no_other_paths else ("persistent", "levels")):
            if p_ != args.path:
                ms_paths[p_] = pass_ms(lambda p_=p_: b.em_iterations(
                    1, rel_tol=-1.0, max_iters=1 << 30, persistent=p_ == "persistent"), reps=3)
        if args.path != "graph" and not args.no_other_paths:
            g2 = b.em_graph(1, rel_tol=-1.0, max_iters=1 << 30, persistent=False)
            ms_paths["graph"] = pass_ms(lambda: b.launch_graph(g2), reps=3)

    # e2e: public API from host strings / matrix to host results
    e2e = None
    if not args.no_e2e:
        score_candidates(w.newicks, w.rows, w.Q, w.leaf_order, group_sites=G, wide_chunk=CH,
                         wide_pc=PC, device=dev)
        torch.cuda.synchronize(dev)
        tot_iters, t_e2e, h2d, d2h = 0, 0.0, 0, 0
        for _ in range(args.e2e_steps):
            t_a = time.perf_counter()
            res = score_candidates(w.newicks, w.rows, w.Q, w.leaf_order, group_sites=G,
                                   wide_chunk=CH, wide_pc=PC, device=dev)
            t_e2e += time.perf_counter() - t_a
            tot_iters += sum(r.iterations for r in res.results)
            h2d, d2h = res.h2d_bytes, res.d2h_bytes
        e2e = {"value": tot_iters * world / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "seconds_per_step": t_e2e / args.e2e_steps,
               "em_iterations_per_step": tot_iters / args.e2e_steps}

    plain = None
    if not args.no_e2e and args.plain_trees > 0:
        pv = plain_dropin(w, args.plain_trees, dev)
        plain = {"value": pv, "unit": UNIT,
                 "sample": f"{args.plain_trees} candidates one at a time through the "
                           "fastEM_solver mirror (EM to convergence each)"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            def med(n_trees, runs=5):   # one warm-up run, then the median of `runs`
                cpu_sample_port(w, n_trees, 1)
                got = [cpu_sample_port(w, n_trees, 1) for _ in range(runs)]
                return statistics.median(g[0] for g in got), got[0][1]
            v, cores = med(16)
            v1, _ = med(1)   # one tree runs on one core
            cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                   "value_1core": v1, "runs": "median of 5 after a warm-up run",
                   "sample": "16 of the 512 candidates x 1 EM iteration, FP64 C restatement "
                             "of the fastEM path, one tree per core; value_1core: one "
                             "candidate x 1 EM iteration on one core"}
        except Exception as ex:  # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port",
                   "sample": f"unavailable: {ex}"}

    # parity: every candidate's log-likelihood at the starting parameters
    # against the FP64 C restatement (not timed)
    parity = None
    if rank == 0 and not args.no_cpu:
        try:
            from oracle import cpu_port
            ref = cpu_port.loglik(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5)
            rel = np.abs(llh_start / ref - 1.0)
            parity = {"max_rel_err_llh": float(rel.max()), "trees": int(len(ref)),
                      "tolerance": 1e-6, "oracle": "FP64 C restatement of the fastEM path",
                      "at": "starting parameters nu = phi = 0.5, newick branch lengths"}
        except Exception as ex:  # reported, never required
            parity = {"max_rel_err_llh": None, "error": str(ex)}

    # a short Poisson request stream through the continuous-batching server
    # (the serving configuration's request mix; its own run: --serving)
    serving = None
    if rank == 0 and not args.no_serving:
        import copy
        sa = copy.copy(args)
        sa.serve_seconds, sa.serve_drain, sa.serve_pool = args.bench_serve_seconds, 30.0, 8
        try:
            sl = run_serving(sa, emit=False)
            serving = {k: sl[k] for k in (
                "value", "unit", "requests", "completed", "completed_per_s", "em_requests",
                "em_completed_fraction", "unfinished_at_deadline", "offered_rate_per_s",
                "p50_latency_s", "p99_latency_s", "p50_latency_em_s", "p99_latency_em_s",
                "p50_latency_llh_s", "p99_latency_llh_s", "recohorts",
                "em_tree_iterations_launched_per_s", "drain_deadline_s", "capacity")}
            serving["stream_seconds"] = sa.serve_seconds
            serving["value_means"] = "tree-EM-iterations of the answered requests per second"
        except Exception as ex:   # reported, never required
            import traceback
            serving = {"error": str(ex), "where": traceback.format_exc()[-1500:]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "512 NNI candidates of a 1000-leaf Yule tree, 40 sites, "
                                   "M_k~U{5..50}, q~Dir(0.5), nu=0.1, phi=0.15, fastEM semantics",
                       "trees_per_gpu": T, "nodes_per_gpu": nodes, "sites": K,
                       "group_sites": G, "wide_chunk": CH, "wide_pc": PC,
                       "wide_kernel": f"producer/consumer warp pairs, {CH or 8} slots per stage"
                       if PC else "direct per-thread loads" if CH == 0 else
                       f"bulk-staged, {CH} slots per stage",
                       "tile_shape": "autotuned" if tuned else "given",
                       "autotune_ms_per_em_iteration": tuned["ms"] if tuned else None,
                       "l2": "inputs larger than L2 (partials "
                       f"{2 * 4 * b.sizes['part_floats'] / 1e9:.2f} GB)",
                       "parallelism": f"replicas{world}" if world > 1 else "single"},
            "node_site_updates_per_s": nsu,
            "roofline": roof_out,
            "roofline_inside": roof_in,
            "roofline_em_iteration": roof_it,
            "e2e": e2e,
            "plain_gpu_dropin": plain,
            "batched_over_plain": (e2e["value"] / plain["value"]) if (e2e and plain) else None,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": args.steps * (1 if args.path == "persistent" else
                                          b.sizes["n_in_levels"] + b.sizes["n_out_levels"] + 4),
            "path": args.path,
            "ms_per_em_iteration_other_paths": ms_paths,
            "wall_s_timed": t1 - t0,
            "llh_mean": float(np.mean(llh_now)),
            "parity": parity,
            "serving": serving,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
