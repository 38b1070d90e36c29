"""CPU check of the kernels' plan addressing and float32 scaling scheme
(tests/kernel_model.py) against the FP64 oracle, on batches of several
trees, both model modes and every group size."""
import numpy as np
import pytest

from laml_gb300 import problem as PB
from laml_gb300 import synth
from oracle import pmm_oracle as O
from tests.kernel_model import Model


@pytest.mark.parametrize("compat", [True, False])
@pytest.mark.parametrize("G", [8, 16, 32])
def test_kernel_model_matches_oracle(compat, G):
    w = synth.pmm_workload(30, 11, 3, 9, 0.5, 0.1, 0.15, seed=3, n_trees=3)
    ds = PB.dataset_from_rows(w.rows, w.Q, w.leaf_order, compat, G)
    trees = PB.encode_trees(w.newicks, w.leaf_order)
    nu, phi = 0.13, 0.21
    m = Model([ds], trees, [0] * 3, [t.branch_length for t in trees], [nu] * 3, [phi] * 3,
              compat)
    m.run_inside()
    cnt, lr = m.run_outside()
    nb = m.p["tr_node_base"]
    for t in range(3):
        tr = O.parse_tree(w.newicks[t], w.leaf_order)
        enc = O.recode([w.rows[c] for c in w.leaf_order], w.Q, compat=compat)
        es = O.e_step(O.Problem(tr, enc, compat), tr.branch_lengths, nu, phi)
        np.testing.assert_allclose(m.site_llh(t), es.llh_site, rtol=1e-6)
        np.testing.assert_allclose(cnt[nb[t]:nb[t] + trees[t].num_nodes], es.counts,
                                   rtol=1e-4, atol=1e-5)
        np.testing.assert_allclose(lr[nb[t]:nb[t] + trees[t].num_leaves], es.leaf_resp,
                                   rtol=1e-4, atol=1e-5)

