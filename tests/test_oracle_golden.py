"""Pin the FP64 oracle against the reference's own known answers.

* nllh of every literal 3-leaf case in laml_unit_tests/unit_tests_EMSolver.py
  test_1..20, 46 and unit_tests_MLSolver.py test_1..21 (places=5 there);
* the reduced-tree outside identity of unit_tests_EMSolver.py:247-303
  (out0 + log(1-phi) and out1 equal the inside logL of the tree cut at x with
  x observed as 0 / silenced), on tests 21..44 and on the test1 data (test_45);
* the EM fixed point on the test4 data (unit_tests_EMSolver.py:535-602).
"""
import math
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from oracle import pmm_oracle as O  # noqa: E402
from tests.helpers import (known_answers, read_char_matrix, read_prior_csv,  # noqa: E402
                           rows_in_leaf_order, golden_path)

LLH_CASES, OUT_CASES = known_answers()
LLH_CASES = list(LLH_CASES)


def build(newick, msa, Q, compat, order=None):
    tr = O.parse_tree(newick, ordered_leaf_labels=order)
    enc = O.recode(rows_in_leaf_order(tr, msa), Q, compat=compat)
    return O.Problem(tr, enc, compat=compat)


@pytest.mark.parametrize("case", LLH_CASES, ids=[c["name"] for c in LLH_CASES])
def test_known_answer_nllh(case):
    prob = build(case["T"], case["msa"], case["Q"], compat=False)
    llh, _ = O.log_likelihood(prob, prob.tree.branch_lengths, case["nu"], case["phi"])
    assert -llh == pytest.approx(case["true_nllh"], abs=1e-9)


@pytest.mark.parametrize("case", LLH_CASES[:6], ids=[c["name"] for c in LLH_CASES[:6]])
def test_compat_equals_exact_when_priors_sum_to_one(case):
    # with every prior state observed and phi in (0,1), compat differs from exact
    # only by the EPS floors, O(1e-6)
    prob_c = build(case["T"], case["msa"], case["Q"], compat=True)
    prob_e = build(case["T"], case["msa"], case["Q"], compat=False)
    lc, _ = O.log_likelihood(prob_c, prob_c.tree.branch_lengths, 0.1, 0.2)
    le, _ = O.log_likelihood(prob_e, prob_e.tree.branch_lengths, 0.1, 0.2)
    assert lc == pytest.approx(le, rel=1e-4, abs=1e-4)


def _reduced_trees(newick):
    """unit_tests_EMSolver.__get_reduced_trees__ (EMSolver tests 247-264)."""
    root = O.read_newick(newick)
    out = {}
    for v in O.postorder(root):
        if v.is_leaf():
            out[v.label] = newick
    for v in list(O.postorder(root)):
        if v.parent is None or v.is_leaf():
            continue
        kids = v.children
        v.children = []
        out[v.label] = O.write_newick(root)
        v.children = kids
    return out


def _check_outside(T, Q, msa, phi, nu, give_label=False):
    if give_label:
        root = O.read_newick(T)
        i = 0
        for v in O.preorder(root):
            if not v.is_leaf():
                v.label = "I" + str(i)
                i += 1
        T = O.write_newick(root)
    prob = build(T, msa, Q, compat=False)
    es = O.e_step(prob, prob.tree.branch_lengths, nu, phi)
    lab = {l: i for i, l in enumerate(prob.tree.labels)}
    K = prob.enc.chars.shape[1]
    red = _reduced_trees(T)
    for x, tstr in red.items():
        xi = lab[x]
        for code, col, shift in ((0, 0, math.log(1 - phi) if phi < 1 else -np.inf),
                                 (-1, -1, 0.0)):
            msa_x = dict(msa)
            msa_x[x] = [code] * K
            pr = build(tstr, msa_x, Q, compat=False)
            llh_site = O.log_likelihood(pr, pr.tree.branch_lengths, nu, phi)[1]
            est = es.outside[xi, :, col] + shift
            np.testing.assert_allclose(llh_site, est, rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("case", OUT_CASES, ids=[c["name"] for c in OUT_CASES])
def test_outside_identity(case):
    _check_outside(case["T"], case["Q"], case["msa"], case["phi"], case["nu"])


def test_outside_identity_test1_data():
    """unit_tests_EMSolver.py test_45 (150 cells x 60 sites, uniform priors)."""
    T = open(golden_path("test1.tre")).read().strip()
    msa, _ = read_char_matrix(golden_path("test1_charMtrx.txt"), masked_symbol="-")
    k = 60
    Q = []
    for i in range(k):
        Mi = set(msa[x][i] for x in msa if msa[x][i] not in [0, "?"])
        q = {x: 1 / len(Mi) for x in Mi}
        q[0] = 0
        Q.append(q)
    phi, nu = 0.05231954386883335, 0.15877477685098262
    # a subset of cut points keeps this in the CPU budget; every node is
    # covered by the GPU outside test
    root = O.read_newick(T)
    i = 0
    for v in O.preorder(root):
        if not v.is_leaf():
            v.label = "I" + str(i)
            i += 1
    T2 = O.write_newick(root)
    prob = build(T2, msa, Q, compat=False)
    es = O.e_step(prob, prob.tree.branch_lengths, nu, phi)
    lab = {l: j for j, l in enumerate(prob.tree.labels)}
    red = _reduced_trees(T2)
    rng = np.random.default_rng(45)
    keys = sorted(red)
    for x in rng.choice(keys, size=12, replace=False):
        xi = lab[x]
        for code, col, shift in ((0, 0, math.log(1 - phi)), (-1, -1, 0.0)):
            msa_x = dict(msa)
            msa_x[x] = [code] * k
            pr = build(red[x], msa_x, Q, compat=False)
            llh_site = O.log_likelihood(pr, pr.tree.branch_lengths, nu, phi)[1]
            np.testing.assert_allclose(llh_site, es.outside[xi, :, col] + shift,
                                       rtol=1e-9, atol=1e-8)


def _test4():
    T = open(golden_path("test4.tre")).read().strip()
    msa, _ = read_char_matrix(golden_path("test4_charMtrx.txt"), masked_symbol="?")
    Q = read_prior_csv(golden_path("test4_prior.csv"), with_zero_key=True)
    return T, msa, Q


@pytest.mark.slow
def test_exact_em_fixed_point_test4():
    """unit_tests_EMSolver.py test_47: seed 1221, nllh 1007.009158767873
    (relative, 4 places), phi = nu = 0 (4 places)."""
    import random
    T, msa, Q = _test4()
    prob = build(T, msa, Q, compat=False)
    post = O.treeswift_postorder_ids(prob.tree)
    lens = [prob.tree.branch_lengths[i] if prob.tree.has_length[i] else None for i in post]
    rs = random.Random(1221)
    randseed = int(rs.random() * 10000)
    x, nu, phi = O.exact_initials(prob.tree, lens, randseed)
    d = np.empty(len(post))
    d[post] = x
    res = O.em_exact(prob, d, nu, phi)
    nllh = -res.llh
    assert abs(1007.009158767873 - nllh) / 1007.009158767873 < 1e-4
    assert res.phi == pytest.approx(0, abs=1e-4)
    assert res.nu == pytest.approx(0, abs=1e-4)


@pytest.mark.slow
def test_compat_em_fixed_point_test4():
    """unit_tests_fastEMSolver.py test_1: |nllh - 1007.009158767873| < 10 and
    phi, nu ~ 0 (4 places) through the fastEM (compat) semantics, starting
    at nu = phi = 0.5 as fastEM_solver.score_tree does."""
    T, msa, Q = _test4()
    prob = build(T, msa, Q, compat=True)
    res = O.em_compat(prob, prob.tree.branch_lengths, 0.5, 0.5)
    assert abs(1007.009158767873 - (-res.llh)) < 10
    assert res.phi == pytest.approx(0, abs=1e-4)
    assert res.nu == pytest.approx(0, abs=1e-4)
