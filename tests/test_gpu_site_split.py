"""The site split of one tree (laml_gb300/site_split.py) on the device: two
ranks as two processes on one GPU, the all-reduce over gloo on the host (the
ranks' kernels never wait on each other).  Each rank runs the inside and
outside passes on its share of the sites; the reduced counts feed the
device M-step of both ranks.

Against the tree in one batch: every rank holds the same parameters
(bitwise); the log-likelihood after 3 fixed EM iterations equals the
unsplit batch's to 1e-8 relative (the shares group their sites by state count
apart, so FP32 count sums differ in order: parameters to 1e-4; measured
1.1e-9) and the FP64 C restatement's to 1e-6; EM to fastEM's stopping rule stops within one
iteration of the unsplit batch."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _case():
    from laml_gb300 import synth
    return synth.pmm_workload(600, 48, 5, 40, 0.5, 0.1, 0.15, seed=61)


def _worker(rank, world, port, q):
    import torch.distributed as dist

    from laml_gb300 import site_split as SS
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = _case()
    K = len(w.Q)
    shards = SS.site_shards(SS.observed_state_counts(w.rows, w.leaf_order, K), world)
    out = {}
    for key, kw in (("fixed", dict(max_iters=3, rel_tol=-1.0)), ("conv", dict(max_iters=500))):
        em = SS.SiteSplitEM(w.newicks[0], w.rows, w.Q, w.leaf_order, shards[rank], nu=0.5,
                            phi=0.5, compat=True)
        r = em.run(**kw)
        out[key] = (r.llh, r.nu, r.phi, r.iterations, r.branch_lengths.tolist())
        out[key + "_mstats"] = (em.total_missing, em.total_sites)
    q.put((rank, out))
    dist.destroy_process_group()


def test_site_split_two_ranks_on_one_gpu():
    from laml_gb300 import problem as PB
    from oracle import cpu_port
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted([q.get(timeout=600) for _ in range(2)], key=lambda x: x[0])
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    a, b = got[0][1], got[1][1]
    for key in ("fixed", "conv"):
        assert a[key] == b[key]          # both ranks: the same parameters, bitwise
    w = _case()
    nmiss = sum(x == "?" for c in w.leaf_order for x in w.rows[c])
    assert a["fixed_mstats"] == (float(nmiss), 48)
    one = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True)
    r3 = one.run_em(max_iters=3, rel_tol=-1.0, chunk=1)[0]
    llh, nu, phi, ds, _ = cpu_port.em(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5, iters=3)
    s_llh, s_nu, s_phi, s_it, s_d = a["fixed"]
    assert s_it == 3
    assert s_llh == pytest.approx(r3.llh, rel=1e-8)
    assert s_llh == pytest.approx(llh[0], rel=1e-6)
    assert s_nu == pytest.approx(r3.nu, rel=1e-4)
    assert s_phi == pytest.approx(r3.phi, rel=1e-4)
    np.testing.assert_allclose(s_d, r3.branch_lengths, rtol=1e-4, atol=1e-7)
    one = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True)
    rc = one.run_em(max_iters=500)[0]
    c_llh, _, _, c_it, _ = a["conv"]
    assert abs(c_it - rc.iterations) <= 1
    assert c_llh == pytest.approx(rc.llh, rel=1e-7)
