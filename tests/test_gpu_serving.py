"""Continuous batching: requests of mixed tree and site sizes, arriving while
others run, admitted under a small HBM budget; every result equals the same
request run alone (bitwise)."""
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from laml_gb300 import serving as S  # noqa: E402
from laml_gb300 import synth  # noqa: E402


def _requests():
    reqs = []
    rng = np.random.default_rng(5)
    for i in range(10):
        n = int(rng.integers(30, 160))
        K = int(rng.integers(8, 40))
        w = synth.pmm_workload(n, K, 3, 15, 0.5, float(rng.uniform(0, 0.2)),
                               float(rng.uniform(0, 0.3)), seed=100 + i)
        kind = "llh" if i % 3 == 0 else "em"
        reqs.append(S.Request(w.newicks[0], w.rows, w.Q, w.leaf_order, kind=kind,
                              nu=float(rng.uniform(0.05, 0.5)), phi=float(rng.uniform(0.05, 0.5))))
    return reqs


def test_mix_equals_alone():
    reqs = _requests()
    fps = []
    with S.PMMServer(hbm_budget=64 << 20, max_cohort=4, max_cohorts=3) as srv:
        futs = []
        for i, r in enumerate(reqs):
            futs.append(srv.submit(r))
            if i % 4 == 3:
                time.sleep(0.02)     # later arrivals join while earlier cohorts run
        replies = [f.result(timeout=300) for f in futs]
    for r, rep in zip(reqs, replies):
        alone = S.run_alone(r)
        assert rep.result.llh == alone.llh
        assert rep.result.iterations == alone.iterations
        assert rep.result.nu == alone.nu and rep.result.phi == alone.phi
        np.testing.assert_array_equal(rep.result.branch_lengths, alone.branch_lengths)
        assert rep.t_done >= rep.t_admit >= rep.t_submit
        fps.append(rep.latency)
    assert max(fps) < 300


def test_oversized_request_is_refused():
    reqs = _requests()
    with S.PMMServer(hbm_budget=1 << 10) as srv:
        with pytest.raises(ValueError):
            srv.submit(reqs[0])
