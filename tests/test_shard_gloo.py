"""World-size-2 gloo run of the host sharding logic (CPU): every tree lands
in exactly one shard, the gather restores item order, timing is max over
ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from laml_gb300.shard import shard_bounds


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, q):
    import torch.distributed as dist
    from laml_gb300 import shard as S
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    items = list(range(n))
    mine = S.shard(items, rank, world)
    scores = [float(-x) for x in mine]          # stand-in per-tree results
    allv = S.gather_scores(scores, n)
    t = S.max_over_ranks(1.0 + rank)
    q.put((rank, mine, allv, t))
    dist.destroy_process_group()


def test_shard_bounds_cover_exactly_once():
    for n in (0, 1, 7, 512, 513):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = shard_bounds(n, r, world)
                seen += list(range(lo, hi))
            assert seen == list(range(n))


def test_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    n = 11
    ps = [ctx.Process(target=_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert out[0][1] + out[1][1] == list(range(n))
    for _, _, allv, t in out:
        assert allv == [float(-x) for x in range(n)]
        assert t == 2.0


# ---------------------------------------------------------------------------
# the site split of one tree (laml_gb300/site_split.py): each rank's E-step on
# its share of the sites (the FP64 oracle here), one all-reduce, the M-step on
# the sums
# ---------------------------------------------------------------------------
def _site_worker(rank, world, port, q):
    import numpy as np
    import torch
    import torch.distributed as dist

    from laml_gb300 import site_split as SS
    from laml_gb300 import synth
    from oracle import pmm_oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = synth.pmm_workload(70, 23, 3, 14, 0.5, 0.1, 0.15, seed=41)
    K = len(w.Q)
    shards = SS.site_shards(SS.observed_state_counts(w.rows, w.leaf_order, K), world)
    mine = shards[rank]
    rows, Q = SS.sub_matrix(w.rows, w.Q, mine)
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    prob = O.Problem(tr, O.recode([rows[c] for c in w.leaf_order], Q, compat=True), True)
    d, nu, phi = np.maximum(tr.branch_lengths, 1e-6), 0.3, 0.2
    out = []
    for _ in range(3):   # three EM iterations on the reduced statistics
        es = O.e_step(prob, d, nu, phi)
        n = tr.num_leaves
        miss = float(np.sum(prob.enc.chars == O.MISSING))
        loc = np.concatenate([[es.llh, miss, prob.enc.chars.size - miss],
                              es.counts.reshape(-1), es.leaf_resp[:n]])
        t = torch.from_numpy(loc.copy())
        SS.all_reduce_sum(t)
        v = t.numpy()
        llh, M, R = v[0], v[1], v[2]
        N_ = len(tr.parent)
        counts = v[3:3 + 6 * N_].reshape(N_, 6)
        lr = v[3 + 6 * N_:]
        out.append((llh, counts.copy(), lr.copy(), M, R))
        d, nu, phi = O.mstep_compat(counts, float(lr.sum()), R, M, d, nu, phi,
                                    np.ones(N_, bool), False, False)
    q.put((rank, [x.tolist() for x in mine], out, d.tolist(), nu, phi))
    dist.destroy_process_group()


def test_site_shards_cover_and_balance():
    from laml_gb300.site_split import site_shards
    C = [7, 3, 3, 12, 5, 5, 9, 2, 2, 2, 30]
    for world in (1, 2, 3, 4):
        sh = site_shards(C, world)
        assert sorted(int(x) for s in sh for x in s) == list(range(len(C)))
        loads = [sum(C[i] for i in s) for s in sh]
        assert max(loads) - min(loads) <= max(C)


def test_site_split_reduction_two_ranks():
    """The reduced log-likelihood, expected counts and leaf responsibilities
    equal the unsharded E-step's (1e-12: FP64 sums in another order), and
    three EM iterations driven by the sums equal the unsharded EM, with both
    ranks holding the same parameters."""
    import numpy as np

    from laml_gb300 import synth
    from oracle import pmm_oracle as O
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_site_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted([q.get(timeout=300) for _ in range(2)], key=lambda x: x[0])
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(got[0][1] + got[1][1]) == list(range(23))
    w = synth.pmm_workload(70, 23, 3, 14, 0.5, 0.1, 0.15, seed=41)
    tr = O.parse_tree(w.newicks[0], w.leaf_order)
    prob = O.Problem(tr, O.recode([w.rows[c] for c in w.leaf_order], w.Q, compat=True), True)
    d, nu, phi = np.maximum(tr.branch_lengths, 1e-6), 0.3, 0.2
    M = float(np.sum(prob.enc.chars == O.MISSING))
    R = prob.enc.chars.size - M
    for it in range(3):
        es = O.e_step(prob, d, nu, phi)
        for r in range(2):
            llh, counts, lr, Mr, Rr = got[r][2][it]
            assert llh == pytest.approx(es.llh, rel=1e-12)
            np.testing.assert_allclose(counts, es.counts, rtol=1e-12, atol=1e-13)
            np.testing.assert_allclose(lr, es.leaf_resp[:tr.num_leaves], rtol=1e-12,
                                       atol=1e-13)
            assert (Mr, Rr) == (M, R)
        d, nu, phi = O.mstep_compat(es.counts, float(es.leaf_resp.sum()), R, M, d, nu, phi,
                                    np.ones(len(tr.parent), bool), False, False)
    for r in range(2):
        np.testing.assert_allclose(got[r][3], d, rtol=1e-9)
        assert got[r][4] == pytest.approx(nu, rel=1e-9)
        assert got[r][5] == pytest.approx(phi, rel=1e-9)
    assert got[0][3] == got[1][3] and got[0][4] == got[1][4]
