"""The C restatement (oracle/pmm_oracle.c) equals the NumPy oracle."""
import numpy as np

from laml_gb300 import synth
from oracle import cpu_port
from oracle import pmm_oracle as O


def test_c_port_matches_numpy_oracle():
    w = synth.pmm_workload(40, 12, 3, 12, 0.5, 0.1, 0.15, seed=3, n_trees=3)
    llh, nu, phi, ds, _ = cpu_port.em(w.newicks, w.rows, w.Q, w.leaf_order, 0.5, 0.5, iters=3)
    for i in range(3):
        tr = O.parse_tree(w.newicks[i], w.leaf_order)
        enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, True)
        r = O.em_compat(O.Problem(tr, enc, True), tr.branch_lengths, 0.5, 0.5, max_iters=3,
                        stop=-1)
        assert abs(llh[i] / r.llh - 1) < 1e-12
        assert abs(nu[i] / r.nu - 1) < 1e-10
        assert abs(phi[i] / r.phi - 1) < 1e-12
        np.testing.assert_allclose(ds[i], r.d, rtol=1e-10)
