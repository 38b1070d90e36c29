"""Shared test helpers: golden-fixture loading and reference-format readers."""
import json
import os

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _undict(v):
    if isinstance(v, dict) and "__dict__" in v:
        return {_undict(k): _undict(x) for k, x in v["__dict__"]}
    if isinstance(v, list):
        return [_undict(x) for x in v]
    return v


def known_answers():
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        d = json.load(f)
    return ({**c, "Q": _undict(c["Q"]), "msa": _undict(c["msa"])} for c in d["llh"]), \
        [{**c, "Q": _undict(c["Q"]), "msa": _undict(c["msa"])} for c in d["outside"]]


def ultrametric_cases():
    """The ultrametric brute-force known answers (unit_tests_TopoSearch.py)."""
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        d = json.load(f)
    return [{**c, "Q": _undict(c["Q"]), "msa": _undict(c["msa"])} for c in d["ultrametric"]]


def rooted_topologies(leaves):
    """Every rooted binary topology on ``leaves`` as a newick string (15 for
    four leaves), children sorted so each topology appears once."""
    import itertools
    if len(leaves) == 1:
        return [leaves[0]]
    out = set()
    first, rest = leaves[0], list(leaves[1:])
    for k in range(len(rest)):
        for comb in itertools.combinations(rest, k):
            left = [first, *comb]
            right = [x for x in rest if x not in comb]
            for a in rooted_topologies(left):
                for b in rooted_topologies(right):
                    out.add("(" + ",".join(sorted([a, b])) + ")")
    return sorted(out)


def read_char_matrix(path, masked_symbol="?"):
    """sequence_lib.read_charMtrx (sequence_lib.py:139-175): first row holds
    site names; '?', the masked symbol, letters and negative integers become
    '?'."""
    msa = {}
    with open(path) as f:
        sites = f.readline().strip().split(",")
        if sites[0] == "cell_name" or "cell" in sites[0]:
            sites = sites[1:]
        for line in f:
            parts = line.strip().split(",")
            if len(parts) < 2:
                continue
            seq = []
            for x in parts[1:]:
                miss = x in ("?", "-", masked_symbol) or x.isalpha()
                if not miss:
                    try:
                        miss = int(x) < 0
                    except ValueError:
                        miss = False
                seq.append("?" if miss else int(x))
            msa[parts[0]] = seq
    return msa, sites


def read_prior_csv(path, with_zero_key=False, k=None):
    """read_priors CSV branch (sequence_lib.py:324-355); ``with_zero_key``
    mimics unit_tests_EMSolver.py:546-560 (each site dict seeded with {0: 0})."""
    Q = []
    cur = None
    seen = []
    with open(path) as f:
        for line in f:
            s, st, p = line.strip().split(",")
            s = int(s)
            if s not in seen:
                seen.append(s)
                cur = {0: 0.0} if with_zero_key else {}
                Q.append(cur)
            cur[int(st)] = float(p)
    return Q


def rows_in_leaf_order(tree, msa):
    return [msa[tree.labels[i]] for i in range(tree.num_leaves)]


def golden_path(name):
    return os.path.join(GOLDEN, name)
