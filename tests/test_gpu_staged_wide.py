"""The three kernels of the wide levels (more than 8192 items) against each
other and the oracle: per-thread row loads (laml_batch.wide_chunk = 0),
bulk-staged rows (k_items_ws: per-warp shared-memory stages filled by
cp.async.bulk, 8 or 16 state slots per stage) and producer/consumer warp
pairs (k_items_pc, laml_batch.wide_pc: a producer warp bulk-copies rows and
per-site scalars for its consumer warp).  Every thread's arithmetic is
the same in the same order, so an E-step (log-likelihoods, count partials,
posteriors, partial rows and scalars) and three EM iterations agree
bitwise; both match the FP64 C restatement."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from laml_gb300 import problem as PB  # noqa: E402
from laml_gb300 import synth  # noqa: E402
from oracle import cpu_port  # noqa: E402

KEYS = ("tr_llh", "llh_site", "cnt_part", "in_part", "out_part", "post0", "post1", "in_h", "in_x",
        "in_dot", "out_h", "out_x")


def _case():
    return synth.pmm_workload(1000, 40, 5, 50, 0.5, 0.1, 0.15, 3, n_trees=24, nni=True)


def _run(w, G, ch, pc=False):
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, group_sites=G,
                      nu=0.1, phi=0.15, want_post=True)
    b.wide_chunk = ch
    b.wide_pc = pc
    assert max(np.diff(b._h_in_off)) > 8192
    for k in ("in_part", "out_part", "in_dot", "post0", "post1", "cnt_part"):
        b.work[k].fill_(float("nan"))   # words no kernel writes stay NaN in every run
    for k in ("in_h", "in_x", "out_h", "out_x"):
        b.work[k].fill_(-12345)
    b.e_step(want_post=True)
    torch.cuda.synchronize()
    b.check_device_error()
    out = {k: b.work[k].cpu().numpy() for k in KEYS}
    r = b.run_em(max_iters=3, rel_tol=-1.0, chunk=1)
    b.check_device_error()
    out["em_llh"] = np.array([x.llh for x in r])
    out["em_d"] = np.concatenate([x.branch_lengths for x in r])
    return out


@pytest.mark.parametrize("G", [8, 16, 32])
def test_staged_wide_equals_direct_wide_bitwise(G):
    w = _case()
    direct = _run(w, G, 0)
    for ch in (8, 16):
        staged = _run(w, G, ch)
        for k, a in staged.items():
            np.testing.assert_array_equal(a, direct[k], err_msg=f"{k} (slots per stage {ch})")


@pytest.mark.parametrize("G", [8, 16, 32])
def test_pc_wide_equals_direct_wide_bitwise(G):
    w = _case()
    direct = _run(w, G, 0)
    for ch in (8, 16):
        pc = _run(w, G, ch, pc=True)
        for k, a in pc.items():
            np.testing.assert_array_equal(a, direct[k], err_msg=f"{k} (pc, slots per stage {ch})")


def test_pc_wide_matches_oracle():
    w = _case()
    ref = cpu_port.loglik(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5)
    lr, nu, phi, ds, _ = cpu_port.em(w.newicks[:4], w.rows, w.Q, w.leaf_order, 0.5, 0.5,
                                     iters=3)
    for G in (8, 16, 32):
        b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, group_sites=G,
                          nu=0.5, phi=0.5)
        b.wide_pc = True
        np.testing.assert_allclose(b.log_likelihood(), ref, rtol=1e-6)
        r = b.run_em(max_iters=3, rel_tol=-1.0, chunk=1)
        for t in range(4):
            assert r[t].llh == pytest.approx(lr[t], rel=1e-6)
            assert r[t].nu == pytest.approx(nu[t], rel=1e-3)


def test_staged_wide_matches_oracle():
    w = _case()
    ref = cpu_port.loglik(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5)
    lr, nu, phi, ds, _ = cpu_port.em(w.newicks[:4], w.rows, w.Q, w.leaf_order, 0.5, 0.5,
                                     iters=3)
    for G in (8, 16, 32):
        b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, group_sites=G,
                          nu=0.5, phi=0.5)
        b.wide_chunk = 16
        np.testing.assert_allclose(b.log_likelihood(), ref, rtol=1e-6)
        r = b.run_em(max_iters=3, rel_tol=-1.0, chunk=1)
        for t in range(4):
            assert r[t].llh == pytest.approx(lr[t], rel=1e-6)
            assert r[t].nu == pytest.approx(nu[t], rel=1e-3)
