"""The annotation file from the GPU's exact-model E-step against the
reference's own output for examples/example1 (laml_libs/runner.py:391-430;
fixtures and the oracle path in tests/test_annotate.py).

The GPU's posteriors and expected counts are FP32: an entry whose FP64 value
lies within 1e-5 of a rounding boundary of the output (2 decimals for the
posteriors, 3 for the branch lengths) may print the neighbouring value.
Every other character equals the reference's; the ties are counted and
bounded."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from laml_gb300 import annotate as A  # noqa: E402
from tests.test_annotate import example1, oracle_estep  # noqa: E402

TIE = 1e-5


def _near_boundary(x, decimals):
    s = x * 10 ** decimals
    return abs(s - np.floor(s) - 0.5) * 10 ** -decimals < TIE


def test_gpu_annotations_match_reference_output():
    ex = example1()
    et, rows, d, es = oracle_estep(ex)
    tree_line, lines = A.annotate(ex["newick"], ex["msa"], ex["Q"], ex["nu"], ex["phi"],
                                  branch_lengths=d)
    ref = ex["ref"]
    assert len(lines) == len(ref) - 1 == 500
    _, order = A.az_labels(et, rows)
    p0, p1 = np.exp(es.post0), np.exp(es.post1)
    ties = 0
    for k, ((name, s), r) in enumerate(zip(lines, ref[1:])):
        rn, rs = r.split(",", 1)
        assert name == rn
        if s == rs:
            continue
        u = order[k - 1]   # line 0 is the added root I0
        got, want = s.split(","), rs.split(",")
        assert len(got) == len(want)
        for c, (g, w) in enumerate(zip(got, want)):
            if g != w:
                assert _near_boundary(p0[u, c], 2) or _near_boundary(p1[u, c], 2) or \
                    _near_boundary(1 - round(p0[u, c], 2) - round(p1[u, c], 2), 2), \
                    (name, c, g, w, p0[u, c], p1[u, c])
                ties += 1
    # the tree line: names and shape equal; lengths equal except 3-decimal ties
    mut = es.counts[:, 1] + es.counts[:, 2] + es.counts[:, 4]
    if tree_line != ref[0]:
        import re
        tok = re.compile(r"([^,():;]+):([0-9.e-]+)")
        gl, rl = tok.findall(tree_line), tok.findall(ref[0])
        assert [a for a, _ in gl] == [a for a, _ in rl]
        lab = {et.labels[u]: u for u in range(et.num_nodes)}
        for (a, x), (_, y) in zip(gl, rl):
            if x != y:
                assert _near_boundary(mut[lab[a]], 3), (a, x, y, mut[lab[a]])
                ties += 1
    assert ties <= 5, ties
