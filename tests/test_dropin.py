"""The reference-facing mirror: fast_em.{calculations,laml,phylogeny} and the
fastEM_solver class, exercised the way the reference's own unit tests use
them (laml_unit_tests/unit_tests_fastEMSolver.py, unit_tests_EMSolver.py
test_47/48, unit_tests_MLSolver.py)."""
import numpy as np
import pytest

from laml_gb300 import fastEM_solver as FS
from laml_gb300.fast_em import phylogeny as PH
from oracle import pmm_oracle as O
from tests.helpers import (golden_path, known_answers, read_char_matrix, read_prior_csv,
                           rows_in_leaf_order)


def _test4(zero_key=False):
    T = open(golden_path("test4.tre")).read().strip()
    msa, _ = read_char_matrix(golden_path("test4_charMtrx.txt"))
    Q = read_prior_csv(golden_path("test4_prior.csv"), with_zero_key=zero_key)
    return T, msa, Q


# ---------------------------------------------------------------- CPU only
def test_parse_tree_and_parse_data_match_reference_encoding():
    T, msa, Q = _test4()
    pt = FS.parse_tree(T)
    ot = O.parse_tree(T)
    assert pt["relabeling_vector"] == ot.labels
    assert pt["num_leaves"] == ot.num_leaves
    np.testing.assert_array_equal(pt["branch_lengths"], ot.branch_lengths)
    ph = FS.parse_data(pt, {"charMtrx": msa}, {"Q": Q})
    enc = O.recode(rows_in_leaf_order(ot, msa), Q, compat=True)
    np.testing.assert_array_equal(ph.character_matrix, enc.chars)
    np.testing.assert_array_equal(ph.mutation_priors, enc.q.astype(np.float32))
    g = ph.tree
    for u in range(len(ot.parent)):
        assert list(g.successors(u)) == ot.children[u]


def test_write_newick_round_trip():
    T, _, _ = _test4()
    et = FS.encode_newick(T)
    nw = FS.write_newick(et)
    et2 = FS.encode_newick(nw)
    assert et2.labels == et.labels
    np.testing.assert_array_equal(et2.child0, et.child0)
    np.testing.assert_allclose(et2.branch_length, et.branch_length)


def test_parse_newick_mirror():
    g, n = PH.parse_newick("((a:1,b:2):0.5,c:3):0.25;")
    assert n == 3 and g.number_of_nodes() == 5
    assert [g.nodes[i]["label"] for i in range(3)] == ["c", "b", "a"]


# ---------------------------------------------------------------- GPU
@pytest.mark.gpu
def test_fastem_solver_score_tree_test4():
    """unit_tests_fastEMSolver.py test_1/test_48: |nllh - 1007.009...| < 10,
    phi, nu ~ 0 (4 places)."""
    T, msa, Q = _test4()
    pt = FS.parse_tree(T)
    ph = FS.parse_data(pt, {"charMtrx": msa}, {"Q": Q})
    order = pt["relabeling_vector"][:pt["num_leaves"]]
    solver = FS.fastEM_solver([T], {"charMtrx": msa, "ordered_leaf_labels": [order],
                                    "charMtrx_recode": [ph.character_matrix]},
                              {"Q": Q, "Q_recode": [ph.mutation_priors]}, {"phi": 0, "nu": 0})
    score, status = solver.score_tree({'ultra_constr': False, 'fixed_phi': None,
                                       'fixed_nu': None, 'fixed_brlen': None,
                                       'nodes_to_recompute': None})
    assert status == "optimal"
    assert abs(1007.009158767873 + score) < 10
    assert solver.params.phi == pytest.approx(0, abs=1e-4)
    assert solver.params.nu == pytest.approx(0, abs=1e-4)


@pytest.mark.gpu
def test_exact_optimize_test4():
    """unit_tests_EMSolver.py test_47: optimize(initials=1, random_seeds=1221)."""
    T, msa, Q = _test4(zero_key=True)
    solver = FS.fastEM_solver([T], {"charMtrx": msa}, {"Q": Q}, {"phi": 0, "nu": 0})
    nllh, status = solver.optimize(initials=1, random_seeds=1221, verbose=-1,
                                   ultra_constr=False)
    assert abs(1007.009158767873 - nllh) / 1007.009158767873 < 1e-4
    assert solver.params.phi == pytest.approx(0, abs=1e-4)
    assert solver.params.nu == pytest.approx(0, abs=1e-4)


@pytest.mark.gpu
def test_final_optimization_runs_exact_em():
    """unit_tests_EMSolver.py test_48 through score_tree's final_optimization
    branch (fastEM_solver.py:295-297)."""
    T, msa, Q = _test4(zero_key=True)
    solver = FS.fastEM_solver([T], {"charMtrx": msa}, {"Q": Q}, {"phi": 0, "nu": 0})
    score, _ = solver.score_tree({'ultra_constr': False, 'fixed_phi': None, 'fixed_nu': None,
                                  'fixed_brlen': None, 'final_optimization': True})
    assert abs(1007.009158767873 + score) / 1007.009158767873 < 1e-4


@pytest.mark.gpu
def test_negative_llh_known_answers():
    """unit_tests_MLSolver.py / EMSolver.py test_1..20: negative_llh()."""
    cases, _ = known_answers()
    for case in cases:
        solver = FS.fastEM_solver([case["T"]], {"charMtrx": case["msa"]}, {"Q": case["Q"]})
        solver.params = FS.Params(case["nu"], case["phi"])
        assert solver.negative_llh() == pytest.approx(case["true_nllh"], abs=1e-5), case["name"]


@pytest.mark.gpu
def test_fast_em_calculations_mirror():
    from laml_gb300.fast_em import calculations as calc
    from laml_gb300.fast_em.laml import EMOptimizer
    T, msa, Q = _test4()
    pt = FS.parse_tree(T)
    ph = FS.parse_data(pt, {"charMtrx": msa}, {"Q": Q})
    g = ph.tree
    N = g.number_of_nodes()
    n = ph.num_leaves
    leaves = np.arange(n)
    post = O._postorder_ids(O.parse_tree(T))
    ip = np.array([[u, 0] for u in post if u >= n])
    ipc = np.array([list(g.successors(int(u))) for u in ip[:, 0]])
    d = pt["branch_lengths"]
    mp = np.array([0.1, 0.2])
    llh = calc.compute_log_likelihood(d, ph.mutation_priors, leaves, ip, ipc, None, None, None,
                                      mp, ph.character_matrix, n)
    prob = O.Problem(O.parse_tree(T), O.recode(rows_in_leaf_order(O.parse_tree(T), msa), Q),
                     True)
    es = O.e_step(prob, d, 0.1, 0.2)
    assert llh == pytest.approx(es.llh, rel=1e-6)
    l2, cnt, lr = calc.compute_E_step(d, ph.mutation_priors, leaves, ip, ipc, None, None, None,
                                      mp, ph.character_matrix, n)
    np.testing.assert_allclose(cnt, es.counts, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(lr, es.leaf_resp, rtol=1e-4, atol=1e-5)
    opt = EMOptimizer(ph.mutation_priors, ph.character_matrix)
    out = opt.optimize(g, d, 0.5, 0.5, np.ones(N, bool))
    ref = O.em_compat(prob, d, 0.5, 0.5)
    assert -out["nllh"] == pytest.approx(ref.llh, rel=1e-6)
    assert abs(out["em_iterations"] - ref.iterations) <= 1
