"""CPU checks of the C ABI: the library loads, exports every symbol declared
in include/laml_gb300.h, and its host encoders agree with the oracle
bit-for-bit (node numbering, recoding, priors)."""
import os
import re

import numpy as np
import pytest

from laml_gb300 import _native as N
from laml_gb300 import encoding as E
from laml_gb300 import synth
from oracle import pmm_oracle as O
from tests.helpers import golden_path, read_char_matrix, read_prior_csv, rows_in_leaf_order

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "laml_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(laml_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol():
    import ctypes
    lib = ctypes.CDLL(N.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(N.EXPORTS), set(syms) - set(N.EXPORTS)


def test_batch_struct_matches_header():
    """Field order of laml_batch in the ctypes mirror equals the header."""
    src = open(HEADER).read()
    body = src[src.index("typedef struct laml_batch {"):src.index("} laml_batch;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = []
    for line in body.splitlines()[1:]:
        line = line.strip()
        if not line:
            continue
        decl = line.rstrip(";")
        parts = decl.split(None, 1) if not decl.startswith("const") else decl.split(None, 2)[1:]
        rest = parts[-1] if len(parts) > 1 else parts[0]
        rest = re.sub(r"^(int32_t|int64_t|uint8_t|uint32_t|int16_t|double|float)\s*", "", rest)
        for n in rest.split(","):
            names.append(n.strip().lstrip("*").strip())
    assert names == [n for n, _ in N.BATCH_FIELDS]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_newick_order_matches_parse_tree(seed):
    rng = np.random.default_rng(seed)
    t = synth.yule_tree(40 + seed, rng)
    nw = t.newick()
    order = list(rng.permutation([t.labels[u] for u in t.leaves()]))
    for lo in (None, order):
        et = E.encode_newick(nw, lo)
        ot = O.parse_tree(nw, ordered_leaf_labels=lo)
        assert et.labels == ot.labels
        assert et.num_leaves == ot.num_leaves
        np.testing.assert_array_equal(et.parent, ot.parent)
        for u in range(et.num_nodes):
            ch = ot.children[u]
            assert [et.child0[u], et.child1[u]] == (list(ch) if ch else [-1, -1])
        np.testing.assert_array_equal(et.branch_length, ot.branch_lengths)


def test_newick_unifurcating_root_and_unnamed_nodes():
    nw = "(((a:1,b:2):0.5,c:3):0.25);"
    et = E.encode_newick(nw)
    ot = O.parse_tree(nw)
    assert et.labels == ot.labels
    assert et.num_nodes == 5 and et.num_leaves == 3
    assert et.labels[3] == "node_1"      # preorder index 1 after the dropped root


def test_newick_errors():
    with pytest.raises(N.LamlError):
        E.encode_newick("((a:1,b:1):1,c:1")
    with pytest.raises(N.LamlError) as e:
        E.encode_newick("(a:1,b:1,c:1):1;")
    assert e.value.code == -6
    with pytest.raises(N.LamlError) as e:
        E.encode_newick("((a:1,b:1):1,c:1):1;", ["a", "b"])
    assert e.value.code == -7


@pytest.mark.parametrize("compat", [True, False])
@pytest.mark.parametrize("G", [8, 16, 32])
def test_dataset_recode_matches_oracle(compat, G):
    T = open(golden_path("test4.tre")).read().strip()
    msa, _ = read_char_matrix(golden_path("test4_charMtrx.txt"))
    Q = read_prior_csv(golden_path("test4_prior.csv"), with_zero_key=not compat)
    tr = O.parse_tree(T)
    rows = rows_in_leaf_order(tr, msa)
    enc = O.recode(rows, Q, compat=compat)
    ds = E.encode_dataset(E.char_matrix(rows, exact=not compat), Q, compat=compat, group_sites=G)
    K = len(Q)
    assert ds.n_sites == K and ds.n_sites_pad % G == 0
    for c in range(ds.n_sites_pad):
        o = ds.site_perm[c]
        if o < 0:
            continue
        k = int(enc.k[o])
        assert ds.site_C[c] == k + 2
        g, lane = c // G, c % G
        qv = np.array([ds.q[ds.group_off[g] + j * G + lane] for j in range(2, k + 2)])
        np.testing.assert_array_equal(qv, enc.q[o, :k].astype(np.float32))
        # codes: slot j <-> recoded state j-1
        oc = enc.chars[:, o]
        gc = ds.codes[:, c].astype(np.int64)
        np.testing.assert_array_equal(np.where(gc >= 2, gc - 1, gc), oc)
    assert ds.n_missing == int(np.sum(enc.chars == O.MISSING))


def test_dataset_missing_prior_is_an_error():
    mat = np.array([[1, 2], [0, 3]], np.int32)
    with pytest.raises(N.LamlError) as e:
        E.encode_dataset(mat, [{1: 0.5}, {2: 1.0}], compat=True)
    assert e.value.code == -4


def test_plan_levels():
    rng = np.random.default_rng(5)
    trees = [E.encode_newick(synth.yule_tree(n, rng).newick()) for n in (7, 30, 3)]
    mat = np.zeros((30, 5), np.int32)
    ds = E.encode_dataset(mat, [{1: 1.0}] * 5, compat=True, group_sites=8)
    sizes, arr = E.plan_batch(trees, [0, 0, 0], [ds])
    assert sizes["n_nodes"] == sum(t.num_nodes for t in trees)
    # every internal node appears once per group among the inside items, after its children
    items = arr["in_items"][:2 * sizes["n_in_items"]].reshape(-1, 2)
    lvl = np.empty(sizes["n_nodes"], int)
    off = arr["in_level_off"]
    for l in range(sizes["n_in_levels"]):
        for node, g in items[off[l]:off[l + 1]]:
            lvl[node] = l
    for u in range(sizes["n_nodes"]):
        c0, c1 = arr["nd_c0"][u], arr["nd_c1"][u]
        if c0 >= 0:
            for c in (c0, c1):
                if arr["nd_c0"][c] >= 0:
                    assert lvl[c] < lvl[u]


def test_level_node_lists_give_the_items():
    """plan_batch(items=False): item k of a level with item offset o and c
    nodes is node lnodes[o / NG + (k - o) % c] of group (k - o) // c -- the
    rule laml_plan_descriptors applies on the device."""
    rng = np.random.default_rng(7)
    trees = [E.encode_newick(synth.yule_tree(n, rng).newick()) for n in (9, 40, 3, 17)]
    mat = np.zeros((40, 21), np.int32)
    ds = E.encode_dataset(mat, [{1: 1.0}] * 21, compat=True, group_sites=8)
    sizes, ref = E.plan_batch(trees, [0] * 4, [ds], host_desc=False)
    s2, ln = E.plan_batch(trees, [0] * 4, [ds], host_desc=False, items=False)
    assert "in_items" not in ln and s2 == sizes
    NG = ds.n_groups
    for side, nl in (("in", sizes["n_in_levels"]), ("out", sizes["n_out_levels"])):
        off = ln[f"{side}_level_off"]
        np.testing.assert_array_equal(off, ref[f"{side}_level_off"])
        items = ref[f"{side}_items"][:2 * sizes[f"n_{side}_items"]].reshape(-1, 2)
        nodes = ln[f"{side}_lnodes"]
        for l in range(nl):
            o, c = off[l], (off[l + 1] - off[l]) // NG
            for k in range(off[l], off[l + 1]):
                r = k - o
                assert (nodes[o // NG + r % c], r // c) == tuple(items[k])


def test_item_descriptors_match_plan():
    rng = np.random.default_rng(9)
    trees = [E.encode_newick(synth.yule_tree(n, rng).newick()) for n in (9, 31, 4)]
    mats = [np.zeros((31, 21), np.int32), np.zeros((31, 5), np.int32)]
    dss = [E.encode_dataset(m, [{1: 1.0}] * m.shape[1], compat=True, group_sites=8) for m in mats]
    tree_ds = [0, 1, 0]
    sizes, a = E.plan_batch(trees, tree_ds, dss)
    gbase = a["group_base"]
    for kind in ("in", "out"):
        items = a[f"{kind}_items"][:2 * sizes[f"n_{kind}_items"]].reshape(-1, 2)
        desc = a[f"{kind}_desc"][:12 * len(items)].reshape(-1, 12)
        for (u, g), e in zip(items, desc):
            t = a["nd_tree"][u]
            v, w = a["nd_c0"][u], a["nd_c1"][u]
            assert list(e[:3]) == [u, v, w]
            assert e[3] & 0xffffff == t
            fl = e[3] >> 24
            assert bool(fl & 1) == (a["nd_c0"][v] < 0) and bool(fl & 2) == (a["nd_c0"][w] < 0)
            assert bool(fl & 4) == (a["tr_root"][t] == u)
            assert e[4] == g and e[5] == gbase[tree_ds[t]] + g
            assert e[6] == a["nd_srow"][u] and e[7] * 8 == a["nd_prow"][u]
            for x, ref, sr in ((v, e[8], e[10]), (w, e[9], e[11])):
                if a["nd_c0"][x] < 0:
                    assert ref == a["nd_leafrow"][x]
                else:
                    assert ref * 8 == a["nd_prow"][x] and sr == a["nd_srow"][x]
    gd = a["grp_desc"][:8 * sizes["n_groups_total"]].reshape(-1, 8)
    kp = [d.n_sites_pad for d in dss]
    for d, ds in enumerate(dss):
        for g in range(ds.n_groups):
            e = gd[gbase[d] + g]
            assert e[0] == ds.group_off[g] and e[3] == d and e[5] == ds.n_sites_pad
            assert e[1] == sum(kp[:d]) + g * 8
            assert e[2] == sum(x.row_len for x in dss[:d]) + ds.group_off[g]
            assert e[4] == sum(x.codes.size for x in dss[:d]) and e[6] == ds.n_sites


@pytest.mark.parametrize("nw", [
    "((a:1,b:2):0.5,(c:+1e-3,d:0x1p-2):0.25);",
    "(((a,b),c),d);",
    "( a : 1.5 , [note] b:2 ) ;",
    "((a:1,b:1)n1:1,(c:1e-7,d:1):1)root;",
    "(((a:0.1,b:0.2):0.3,c:1):0.7);",
])
def test_batch_parser_equals_single_tree_parser(nw):
    """laml_newick_encode_batch (flat parser) and laml_newick_encode agree
    on signs, hex lengths, comments, whitespace, unifurcating roots."""
    lo = sorted({ch for ch in "abcd" if ch in nw})
    s = E.encode_newick(nw, lo)
    b = E.encode_newick_batch([nw], lo)[0]
    for f in ("parent", "child0", "child1", "branch_length", "has_length"):
        np.testing.assert_array_equal(getattr(s, f), getattr(b, f), err_msg=f)


def test_batch_parser_errors():
    with pytest.raises(N.LamlError):
        E.encode_newick_batch(["((a,b),(a,c));"], ["a", "b", "c"])     # duplicate leaf
    with pytest.raises(N.LamlError):
        E.encode_newick_batch(["((a,b,c),d);"], ["a", "b", "c", "d"])  # not binary
    with pytest.raises(N.LamlError):
        E.encode_newick_batch(["((a,b),c"], ["a", "b", "c"])           # unbalanced
    with pytest.raises(N.LamlError):
        E.encode_newick_batch(["((((a,b))),c);"], ["a", "b", "c"])     # inner unifurcation


def _expected_items(trees, tree_ds, dss, side):
    """The schedule spelled out: per level (inside: node height; outside:
    depth of the internal parent + 1), groups outermost, then the nodes
    grouped by which children are leaves (bit 0: first child, bit 1: second),
    and within that trees in order and nodes ascending."""
    levels = {}
    base = 0
    for p, t in enumerate(trees):
        N, n = t.num_nodes, t.num_leaves
        h = np.zeros(N, int)
        dep = np.zeros(N, int)
        par = t.parent
        # depth by walking up; height by relaxation until nothing changes
        for u in range(N):
            x, k = u, 0
            while par[x] >= 0:
                x, k = par[x], k + 1
            dep[u] = k
        changed = True
        while changed:
            changed = False
            for u in range(n, N):
                hu = 1 + max(h[t.child0[u]], h[t.child1[u]])
                if hu != h[u]:
                    h[u], changed = hu, True
        ng = dss[tree_ds[p]].n_groups
        for u in range(n, N):
            lv = h[u] if side == "in" else dep[u] + 1
            key = (1 if t.child0[u] < n else 0) | (2 if t.child1[u] < n else 0)
            levels.setdefault(lv, []).append((key, base + u, ng))
        base += N
    out = []
    for lv in sorted(levels):
        nodes = sorted(levels[lv], key=lambda x: x[0])   # stable: trees, nodes ascending
        for g in range(max(d.n_groups for d in dss)):
            out += [(node, g) for _, node, ng in nodes if g < ng]
    return np.asarray(out, np.int32)


@pytest.mark.parametrize("site_counts", [(5, 5), (21, 5), (12, 40)])
def test_item_order_is_the_documented_schedule(site_counts):
    """Uniform group counts take the parallel scatter, mixed ones the general
    loop; both give the documented order."""
    rng = np.random.default_rng(17)
    trees = [E.encode_newick(synth.yule_tree(n, rng).newick()) for n in (9, 31, 4, 17)]
    mats = [np.zeros((31, k), np.int32) for k in site_counts]
    dss = [E.encode_dataset(m, [{1: 1.0}] * m.shape[1], compat=True, group_sites=8)
           for m in mats]
    tree_ds = [0, 1, 0, 1]
    sizes, a = E.plan_batch(trees, tree_ds, dss)
    for side in ("in", "out"):
        got = a[f"{side}_items"][:2 * sizes[f"n_{side}_items"]].reshape(-1, 2)
        np.testing.assert_array_equal(got, _expected_items(trees, tree_ds, dss, side))
