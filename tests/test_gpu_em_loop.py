"""EM to convergence as one graph launch (laml_em_graph_loop_create): a
conditional WHILE node repeats a chunk of EM iterations while some tree is
ACTIVE, fewer than max_chunks chunks ran in the launch and no error is
recorded.  Here the chunk cap ends the loop (a negative tolerance keeps every
tree ACTIVE): the counter is back at zero, a second launch runs the same
number of chunks again, and the trees' state equals the same iterations
issued as per-level launches, bitwise."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from laml_gb300 import _native as N  # noqa: E402
from laml_gb300 import problem as PB  # noqa: E402
from laml_gb300 import synth  # noqa: E402
from laml_gb300.engine import MSTEP_ROUNDS  # noqa: E402


def _batch(w):
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, nu=0.3, phi=0.2)
    b.branch_terms()
    b.inside(update_em=True)
    return b


def test_loop_graph_chunk_cap_relaunch_and_equality():
    w = synth.pmm_workload(60, 12, 3, 10, 0.5, 0.1, 0.15, seed=5, n_trees=3)
    b = _batch(w)
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    h = C.c_void_p()
    N.check(N.lib().laml_em_graph_loop_create(C.byref(b.b), 2, MSTEP_ROUNDS, -1.0, 1000,
                                              b._mflags(None), 3, C.c_void_p(cnt.data_ptr()),
                                              C.byref(h)))
    try:
        b.launch_graph(h)
        torch.cuda.synchronize()
        b.check_device_error()
        assert int(cnt.item()) == 0
        assert (b.work["tr_status"].cpu().numpy() == N.TREE_ACTIVE).all()
        it1 = b.work["tr_iter"].cpu().numpy().copy()
        b.launch_graph(h)
        torch.cuda.synchronize()
        assert int(cnt.item()) == 0
        it2 = b.work["tr_iter"].cpu().numpy()
        np.testing.assert_array_equal(it2, 2 * it1)   # the same 3 chunks again
        c = _batch(w)
        c.em_iterations(12, rel_tol=-1.0, max_iters=1000)   # 2 launches x 3 chunks x 2
        torch.cuda.synchronize()
        for k in ("tr_iter", "tr_llh"):
            np.testing.assert_array_equal(b.work[k].cpu().numpy(), c.work[k].cpu().numpy(), k)
        np.testing.assert_array_equal(b.v["nd_d"].cpu().numpy(), c.v["nd_d"].cpu().numpy())
    finally:
        N.lib().laml_graph_destroy(h)


def test_run_em_default_graph_matches_levels():
    """run_em's default (one launch of the loop graph) against the host-tested
    per-level path, to convergence."""
    w = synth.pmm_workload(80, 14, 3, 10, 0.5, 0.1, 0.15, seed=6, n_trees=4)
    r_graph = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True).run_em(chunk=3)
    r_lv = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True).run_em(
        chunk=3, path="levels")
    for a, c in zip(r_graph, r_lv):
        assert a.llh == c.llh and a.iterations == c.iterations and a.status == c.status
        np.testing.assert_array_equal(a.branch_lengths, c.branch_lengths)
