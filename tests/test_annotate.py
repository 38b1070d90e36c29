"""The posterior annotation file of the runner (laml_libs/runner.py:391-430)
and the input readers (laml_libs/sequence_lib.py:139-175, 324-355) against
the reference's own output for examples/example1 (fixtures in
tests/golden/example1, copied by make_golden.py): the optimised tree
(example1_trees.nwk, written with its lengths divided by the mutation rate,
runner.py:333-345) is restored by multiplying them back; the exact-model
(EM_solver) E-step at the reported phi and nu then gives

* the reported negative log-likelihood, 6987.352449704049 (relative 1e-12);
* the annotated tree line and all 500 node lines of example1_annotations.txt,
  character for character, with the oracle's FP64 posteriors and expected
  counts fed to the writer (``annotate.annotation_lines``)."""
import os

import numpy as np
import pytest

from laml_gb300 import annotate as A
from laml_gb300 import io
from laml_gb300.encoding import encode_newick
from oracle import pmm_oracle as O
from tests.helpers import GOLDEN

EX = os.path.join(GOLDEN, "example1")


def example1():
    msa, sites = io.read_sequences(os.path.join(EX, "character_matrix.csv"))
    Q = io.read_priors(os.path.join(EX, "priors.csv"))
    with open(os.path.join(EX, "example1_params.txt")) as f:
        par = dict(ln.split(": ", 1) for ln in f.read().strip().split("\n"))
    with open(os.path.join(EX, "example1_trees.nwk")) as f:
        nw = f.read().strip()
    with open(os.path.join(EX, "example1_annotations.txt")) as f:
        ref = f.read().strip().split("\n")
    return dict(msa=msa, sites=sites, Q=Q, phi=float(par["Dropout rate"]),
                nu=float(par["Silencing rate"]), rate=float(par["Mutation rate"]),
                nllh=float(par["Negative-llh"].strip("()").split(",")[0]), newick=nw, ref=ref)


def oracle_estep(ex):
    et = encode_newick(ex["newick"])
    tr = O.parse_tree(ex["newick"])
    assert list(tr.labels) == list(et.labels)
    rows = [ex["msa"][et.labels[i]] for i in range(et.num_leaves)]
    prob = O.Problem(tr, O.recode(rows, ex["Q"], compat=False), False)
    d = et.branch_length * ex["rate"]
    return et, rows, d, O.e_step(prob, d, ex["nu"], ex["phi"])


def test_readers_on_example1():
    ex = example1()
    assert len(ex["msa"]) == 250 and len(ex["sites"]) == 30
    assert all(len(v) == 30 for v in ex["msa"].values())
    assert len(ex["Q"]) == 30
    # 22% of the entries are '?' (the shape the 250 x 30 configuration mirrors)
    miss = sum(x == "?" for v in ex["msa"].values() for x in v) / (250 * 30)
    assert 0.15 < miss < 0.3
    assert all(abs(sum(q.values()) - 1.0) < 1e-6 for q in ex["Q"])


def test_example1_annotations_match_reference_output():
    ex = example1()
    et, rows, d, es = oracle_estep(ex)
    assert -es.llh == pytest.approx(ex["nllh"], rel=1e-12)
    mut = es.counts[:, 1] + es.counts[:, 2] + es.counts[:, 4]
    tree_line, lines = A.annotation_lines(et, rows, ex["Q"], np.exp(es.post0),
                                          np.exp(es.post1), mut)
    ref = ex["ref"]
    assert tree_line == ref[0]
    assert len(lines) == len(ref) - 1 == 500
    for (name, s), r in zip(lines, ref[1:]):
        assert name + "," + s == r
