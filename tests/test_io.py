"""Input formats (laml_libs/sequence_lib.py): the character-matrix and prior
readers (139-175, 324-355, the pickle branch 261-322), the writer (78-92),
and the duplicate collapsing around a run (dedup / add_dup, 10-76)."""
import pickle

from laml_gb300 import io
from laml_gb300.tree import read_tree_newick


def _leaves(nw):
    return sorted(v.label for v in read_tree_newick(nw).traverse_leaves())


def test_char_matrix_reader_missing_symbols(tmp_path):
    p = tmp_path / "m.csv"
    p.write_text("cell_name,s1,s2,s3,s4,s5\n"
                 "a,0,3,?,-,2\n"
                 "b,-1,x,7,0,N\n"
                 "c,1,1,1,1,1\n")
    msa, sites = io.read_sequences(str(p))
    assert sites == ["s1", "s2", "s3", "s4", "s5"]
    assert msa["a"] == [0, 3, "?", "?", 2]
    assert msa["b"] == ["?", "?", 7, 0, "?"]   # negative ints and letters are missing
    assert msa["c"] == [1, 1, 1, 1, 1]
    # a masked symbol given by the caller
    p.write_text("cell,r0,r1\na,9,5\nb,5,9\n")
    msa, _ = io.read_sequences(str(p), masked_symbol="9")
    assert msa == {"a": ["?", 5], "b": [5, "?"]}


def test_write_then_read_round_trip(tmp_path):
    cm = {"a": [0, 3, "?"], "b": [1, 0, 2]}
    p = tmp_path / "w.csv"
    io.write_sequences(cm, 3, str(p))
    assert p.read_text().split("\n")[0] == "cell,r0,r1,r2"
    msa, sites = io.read_sequences(str(p))
    assert msa == cm and sites == ["r0", "r1", "r2"]


def test_prior_reader_forms(tmp_path):
    # no header, numeric sites
    p = tmp_path / "q.csv"
    p.write_text("0,1,0.5\n0,2,0.5\n1,1,0.25\n1,4,0.75\n")
    assert io.read_priors(str(p)) == [{1: 0.5, 2: 0.5}, {1: 0.25, 4: 0.75}]
    # a header and 'r'-prefixed site names
    p.write_text("site,state,prob\nr0,1,0.5\nr0,3,0.5\nr1,2,1.0\n")
    assert io.read_priors(str(p)) == [{1: 0.5, 3: 0.5}, {2: 1.0}]
    # pickled {site: {state: prob}}: sites in sorted order, state 0 gets 0
    k = tmp_path / "q.pkl"
    with open(k, "wb") as f:
        pickle.dump({1: {"2": 1.0}, 0: {1: 0.4, 5: 0.6}}, f)
    assert io.read_priors(str(k)) == [{1: 0.4, 5: 0.6, 0: 0}, {2: 1.0, 0: 0}]


def test_dedup_prunes_duplicates_and_add_dup_restores_them():
    cm = {"a": [1, 0, "?"], "b": [1, 2, 0], "c": [1, 0, "?"], "d": [0, 0, 0],
          "e": [1, 0, "?"], "f": [0, 0, 0]}
    nw = "(((a:0.1,b:0.2):0.3,c:0.4):0.5,((d:0.6,e:0.7):0.8,f:0.9):1.0);"
    has, dup_map, cm2, out = io.dedup(cm, [nw])
    assert has and cm2 is cm
    assert dup_map == {"a": ["c", "e"], "d": ["f"]}
    # c, e, f pruned; the unifurcations left behind are suppressed, their
    # lengths added to the child's edge
    assert out == ["((a:0.1,b:0.2):0.8,d:2.4);"]
    back = io.add_dup(out, dup_map)
    assert back == ["((b:0.2,(a:0.005,c:0.005,e:0.005)node_dummy_a:0.1):0.8,"
                    "(d:0.005,f:0.005)node_dummy_d:2.4);"]
    assert _leaves(back[0]) == sorted(cm)


def test_dedup_without_duplicates_returns_the_input():
    cm = {"a": [1, 0], "b": [0, 1], "c": [2, 2]}
    nw = ["((a:1,b:1):1,c:2);"]
    has, dup_map, cm2, out = io.dedup(cm, nw)
    assert not has and dup_map == {} and cm2 is cm and out == nw
