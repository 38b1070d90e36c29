"""Every device-side wait is bounded (laml_batch.wait_limit_ns): a wait
that runs out records LAML_ERR_TIMEOUT in the batch's error word, waits for
its own copies still in flight and returns, and the context stays usable.

The limit set negative makes each wait give up at its first unsatisfied
check -- a wait that runs out on purpose, with no fault, trap or hang: on the
staged per-level kernels (mbarrier phases of the bulk copies, narrow and
wide levels), on the producer/consumer pairs of the wide levels and on the
persistent kernel (its grid barrier).  The next calls on the same context,
with the limit back at its default, match the FP64 C restatement."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from laml_gb300 import _native as N  # noqa: E402
from laml_gb300 import problem as PB  # noqa: E402
from laml_gb300 import synth  # noqa: E402
from oracle import cpu_port  # noqa: E402

ERR_TIMEOUT = -5


def _case():
    return synth.pmm_workload(1000, 40, 5, 50, 0.5, 0.1, 0.15, 3, n_trees=24, nni=True)


def test_staged_level_waits_run_out_then_recover():
    w = _case()
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, nu=0.5, phi=0.5)
    assert max(np.diff(b._h_in_off)) > 8192 and min(np.diff(b._h_in_off)) <= 8192
    b.wide_chunk = 16   # wide levels on the bulk-staged kernels too
    b.b.wait_limit_ns = -1
    b.branch_terms()
    b.inside(update_em=True)
    b.outside()
    torch.cuda.synchronize()
    assert int(b.work["error"].item()) == ERR_TIMEOUT
    b.work["error"].zero_()
    b.b.wait_limit_ns = 0
    llh = b.log_likelihood()
    b.check_device_error()
    ref = cpu_port.loglik(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5)
    np.testing.assert_allclose(llh, ref, rtol=1e-6)


def test_pc_level_waits_run_out_then_recover():
    w = _case()
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, nu=0.5, phi=0.5)
    assert max(np.diff(b._h_in_off)) > 8192
    b.wide_pc = True   # wide levels on producer/consumer warp pairs
    b.b.wait_limit_ns = -1
    b.branch_terms()
    b.inside(update_em=True)
    b.outside()
    torch.cuda.synchronize()
    assert int(b.work["error"].item()) == ERR_TIMEOUT
    b.work["error"].zero_()
    b.b.wait_limit_ns = 0
    llh = b.log_likelihood()
    b.check_device_error()
    ref = cpu_port.loglik(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5)
    np.testing.assert_allclose(llh, ref, rtol=1e-6)


def test_persistent_grid_barrier_runs_out_then_recovers():
    w = _case()
    b = PB.make_batch(w.newicks[:4], w.rows, w.Q, w.leaf_order, compat=True)
    b.branch_terms()
    b.inside(update_em=True)
    b.b.wait_limit_ns = -1
    b.em_iterations(1, rel_tol=-1.0, persistent=True)
    torch.cuda.synchronize()
    assert int(b.work["error"].item()) == ERR_TIMEOUT
    # the same context: a fresh run to 3 iterations on the persistent kernel
    c = PB.make_batch(w.newicks[:4], w.rows, w.Q, w.leaf_order, compat=True)
    r = c.run_em(max_iters=3, rel_tol=-1.0, chunk=1, path="persistent")
    c.check_device_error()
    llh, nu, phi, ds, _ = cpu_port.em(w.newicks[:4], w.rows, w.Q, w.leaf_order, 0.5, 0.5,
                                      iters=3)
    for t in range(4):
        assert r[t].llh == pytest.approx(llh[t], rel=1e-6)
