"""Benchmark: batched PMM EM on 512 NNI candidates of a 1000-leaf Yule tree.

Workload (seeded synthetic data, the shapes of the batched NNI-scoring
configuration): one 1,000-leaf Yule tree (branch lengths ~ Exp(mean 0.1),
floor 0.006) and 511 random NNI neighbours; a shared 40-site matrix simulated
under PMM (nu = 0.1, phi = 0.15, M_k ~ U{5..50}, q ~ Dirichlet(0.5)); fastEM
(compat) semantics.

A step is one EM iteration over the whole batch (outside + expected counts ->
M-step -> inside + log-likelihood), one persistent cooperative launch.
``value`` is tree-EM-iterations per second with the batch resident in HBM
(convergence disabled so every step does the full work; the partial buffers,
~3.7 GB, are far larger than L2, so no flush is needed).  ``e2e`` scores the
same 512 candidates through the public API from host newick strings and the
host character matrix to converged results back on the host, timed by wall
clock with the copies inside.

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


def algorithmic_bytes(b):
    """Bytes one fused EM iteration must move (the layout's own words):
    inside reads each internal child row and writes each internal row (2A);
    outside reads the parent's outside row, the sibling's and the node's own
    inside rows and writes the node's outside row (4A); per internal
    (node, site) scalars: 24 B inside + 40 B outside; leaf codes 2 B per leaf
    site read three times; count partials 32 B per (node, group) written and
    read back by the M-step; 8 B per node of branch lengths in the M-step."""
    s = b.sizes
    A = 4 * s["part_floats"]
    leaf_sites = sum(t.num_leaves * b.datasets[b.tree_ds[p]].n_sites_pad
                     for p, t in enumerate(b.trees))
    return (6 * A + 64 * s["scalar_len"] + 6 * leaf_sites + 2 * 4 * s["count_floats"]
            + 8 * 4 * s["n_nodes"])


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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--group-sites", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--ref-trees", type=int, default=16)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--levels", action="store_true",
                    help="one launch per tree level instead of the persistent kernel")
    ap.add_argument("--trees", type=int, default=512,
                    help="use the first N candidates (smaller cases for profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

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
    G = args.group_sites or tune.pick_group_sites(w)
    stream = torch.cuda.Stream(dev)
    with torch.cuda.stream(stream):
        b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, group_sites=G,
                          nu=0.5, phi=0.5, device=dev, stream=stream)
        b.branch_terms()
        b.inside(update_em=True)
    T = b.T
    nodes = b.sizes["n_nodes"]
    K = b.datasets[0].n_sites

    def step():
        b.em_iterations(1, rel_tol=-1.0, max_iters=1 << 30, persistent=not args.levels)

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
    launch_ms = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[-1])
    if world > 1:
        tt = torch.tensor([total_ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
    ms = total_ms / args.steps
    value = T * world * args.steps / (total_ms / 1e3)
    nsu = 2.0 * nodes * K * world * args.steps / (total_ms / 1e3)
    bytes_it = algorithmic_bytes(b)
    avg_launch_s = statistics.mean(launch_ms) / 1e3
    peak, peak_kind = peaks()
    achieved = bytes_it / avg_launch_s / 1e9
    llh_now = b.work["tr_llh"].cpu().numpy()

    # e2e: public API from host strings / matrix to host results
    e2e = None
    if not args.no_e2e:
        score_candidates(w.newicks, w.rows, w.Q, w.leaf_order, group_sites=G, device=dev)
        torch.cuda.synchronize(dev)
        tot_iters, t_e2e, h2d, d2h = 0, 0.0, 0, 0
        for _ in range(args.e2e_steps):
            t_a = time.perf_counter()
            res = score_candidates(w.newicks, w.rows, w.Q, w.leaf_order, group_sites=G,
                                   device=dev)
            t_e2e += time.perf_counter() - t_a
            tot_iters += sum(r.iterations for r in res.results)
            h2d, d2h = res.h2d_bytes, res.d2h_bytes
        e2e = {"value": tot_iters * world / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "seconds_per_step": t_e2e / args.e2e_steps,
               "em_iterations_per_step": tot_iters / args.e2e_steps}

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            v, cores = cpu_sample_port(w, 16, 1)
            cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": "16 of the 512 candidates x 1 EM iteration, FP64 C restatement "
                             "of the fastEM path, one tree per core"}
        except Exception as ex:  # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port",
                   "sample": f"unavailable: {ex}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "512 NNI candidates of a 1000-leaf Yule tree, 40 sites, "
                                   "M_k~U{5..50}, q~Dir(0.5), nu=0.1, phi=0.15, fastEM semantics",
                       "trees_per_gpu": T, "nodes_per_gpu": nodes, "sites": K,
                       "group_sites": G, "l2": "inputs larger than L2 (partials "
                       f"{2 * 4 * b.sizes['part_floats'] / 1e9:.2f} GB)",
                       "parallelism": f"replicas{world}" if world > 1 else "single"},
            "node_site_updates_per_s": nsu,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None,
                         "kernel": "k_items (per level)" if args.levels else "k_em_persistent",
                         "bytes_per_launch": bytes_it,
                         "peak_kind": peak_kind},
            "e2e": e2e,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": args.steps * (1 if not args.levels else
                                          b.sizes["n_in_levels"] + b.sizes["n_out_levels"] + 4),
            "wall_s_timed": t1 - t0,
            "llh_mean": float(np.mean(llh_now)),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
