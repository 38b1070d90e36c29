"""Host logic of the batched API and of the planner's item lists (no
device): the pipeline's part bounds, and plan_batch's level node lists
falling back to (node, group) items when the datasets differ in group
count."""
import numpy as np

from laml_gb300 import encoding as E
from laml_gb300 import synth
from laml_gb300.api import part_bounds


def test_part_bounds_cover_in_growing_shares():
    for T in (1, 2, 7, 256, 512, 1000):
        for parts in range(1, min(T, 6) + 1):
            b = part_bounds(T, parts)
            assert b[0] == 0 and b[-1] == T and len(b) == parts + 1
            sizes = np.diff(b)
            assert (sizes >= 0).all() and sizes.sum() == T
            if T >= 64:   # shares 1 : 2 : ... : parts, up to rounding
                w = np.arange(1, parts + 1)
                np.testing.assert_allclose(sizes, T * w / w.sum(), atol=1.0)
    assert part_bounds(512, 2) == [0, 170, 512]


def test_level_lists_fall_back_to_items_across_group_counts():
    rng = np.random.default_rng(3)
    trees = [E.encode_newick(synth.yule_tree(n, rng).newick()) for n in (12, 9)]
    mats = [np.zeros((12, 13), np.int32), np.zeros((9, 29), np.int32)]
    dss = [E.encode_dataset(m, [{1: 1.0}] * m.shape[1], compat=True, group_sites=8)
           for m in mats]
    assert dss[0].n_groups != dss[1].n_groups
    _, arr = E.plan_batch(trees, [0, 1], dss, host_desc=False, items=False)
    assert "in_items" in arr and "in_lnodes" not in arr
    _, one = E.plan_batch(trees, [0, 0], dss[:1], host_desc=False, items=False)
    assert "in_lnodes" in one and "in_items" not in one
