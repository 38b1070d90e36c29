"""The bulk-staged wide level kernels (k_items_ws: rows through per-warp
shared-memory stages filled by cp.async.bulk) against the direct wide
kernels (per-thread global loads, LAML_WIDE_KERNEL=direct, run in a child
process since the choice is read once per process): every thread's
arithmetic is the same in the same order, so an E-step (log-likelihoods,
count partials, posteriors, partial rows) and three EM iterations agree
bitwise; and against the FP64 oracle."""
import os
import subprocess
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RUN = r'''
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
from laml_gb300 import problem as PB, synth
out = {}
for G in (8, 16, 32):
    w = synth.pmm_workload(1000, 40, 5, 50, 0.5, 0.1, 0.15, 3, n_trees=24, nni=True)
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, group_sites=G,
                      nu=0.1, phi=0.15, want_post=True)
    assert max(np.diff(b._h_in_off)) > 8192
    for k in ("in_part", "out_part", "in_dot", "post0", "post1", "cnt_part"):
        b.work[k].fill_(float("nan"))   # words no kernel writes stay NaN in both runs
    for k in ("in_h", "in_x", "out_h", "out_x"):
        b.work[k].fill_(-12345)
    b.e_step(want_post=True)
    torch.cuda.synchronize()
    b.check_device_error()
    for k in ("tr_llh", "llh_site", "cnt_part", "in_part", "out_part", "post0", "post1",
              "in_h", "in_x", "in_dot", "out_h", "out_x"):
        out[f"{G}_{k}"] = b.work[k].cpu().numpy()
    r = b.run_em(max_iters=3, rel_tol=-1.0, chunk=1)
    out[f"{G}_em_llh"] = np.array([x.llh for x in r])
    out[f"{G}_em_d"] = np.concatenate([x.branch_lengths for x in r])
np.savez(sys.argv[2], **out)
'''


def _run(tmp_path, env_extra):
    script = tmp_path / "run.py"
    script.write_text(_RUN)
    out = tmp_path / f"out_{len(env_extra)}.npz"
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, str(script), ROOT, str(out)], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return np.load(out)


def test_staged_wide_equals_direct_wide_bitwise(tmp_path):
    staged = _run(tmp_path, {})
    direct = _run(tmp_path, {"LAML_WIDE_KERNEL": "direct"})
    for k in staged.files:
        a, c = staged[k], direct[k]
        assert a.shape == c.shape, k
        # words neither kernel writes (slots past a site's state count,
        # padding lanes) hold the same fill in both runs
        np.testing.assert_array_equal(a, c, err_msg=k)


def test_staged_wide_matches_oracle():
    from laml_gb300 import problem as PB
    from laml_gb300 import synth
    from oracle import cpu_port
    w = synth.pmm_workload(1000, 40, 5, 50, 0.5, 0.1, 0.15, 3, n_trees=24, nni=True)
    for G in (8, 16, 32):
        b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, group_sites=G,
                          nu=0.5, phi=0.5)
        llh = b.log_likelihood()
        ref = cpu_port.loglik(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5)
        np.testing.assert_allclose(llh, ref, rtol=1e-6)
        r = b.run_em(max_iters=3, rel_tol=-1.0, chunk=1)
        lr, nu, phi, ds, _ = cpu_port.em(w.newicks[:4], w.rows, w.Q, w.leaf_order, 0.5, 0.5,
                                         iters=3)
        for t in range(4):
            assert r[t].llh == pytest.approx(lr[t], rel=1e-6)
            assert r[t].nu == pytest.approx(nu[t], rel=1e-3)
