"""Build device batches from the reference's in-memory data forms.

``rows``: dict cell label -> list of int | '?'  (data['charMtrx'] of the
reference, laml_libs/sequence_lib.py:139-175);
``Q``: list of {state: prob} per site (prior['Q'], sequence_lib.py:233-363);
``leaf_order``: the leaf labels in the order the matrix rows are used
(data['ordered_leaf_labels'], fastEM_solver.py:175).
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from .encoding import EncodedTree, char_matrix, encode_dataset, encode_newick
from .engine import DeviceBatch

EPS = 1e-6   # fast_em/calculations.py:9


def dataset_from_rows(rows: dict, Q, leaf_order: Sequence[str], compat: bool = True,
                      group_sites: int = 8):
    mat = char_matrix([rows[c] for c in leaf_order], exact=not compat)
    return encode_dataset(mat, Q, compat=compat, group_sites=group_sites)


def encode_trees(newicks: Sequence[str], leaf_order: Sequence[str]):
    return [encode_newick(nw, leaf_order) for nw in newicks]


def make_batch(newicks: Sequence[str], rows: dict, Q, leaf_order: Sequence[str],
               compat: bool = True, group_sites: int = 8, nu=0.5, phi=0.5,
               d: Optional[Sequence[np.ndarray]] = None, mask=None, fix_nu=None, fix_phi=None,
               want_post: bool = False, clamp: bool = True, device="cuda", stream=None,
               trees: Optional[Sequence[EncodedTree]] = None, dataset=None,
               ultrametric: bool = False) -> DeviceBatch:
    """One dataset shared by every tree.  With ``clamp`` (compat) the starting
    point is prepared as fast_em/laml.py:128-132 does: nu, phi clipped to
    [EPS, 1-EPS] and d floored at EPS."""
    ds = dataset if dataset is not None else dataset_from_rows(rows, Q, leaf_order, compat,
                                                               group_sites)
    trees = trees if trees is not None else encode_trees(newicks, leaf_order)
    if d is None:
        d = [t.branch_length.copy() for t in trees]
    d = [np.asarray(x, np.float64) for x in d]
    nu = np.broadcast_to(np.asarray(nu, np.float64), (len(trees),)).copy()
    phi = np.broadcast_to(np.asarray(phi, np.float64), (len(trees),)).copy()
    if compat and clamp:
        nu = np.clip(nu, EPS, 1 - EPS)
        phi = np.clip(phi, EPS, 1 - EPS)
        d = [np.maximum(x, EPS) for x in d]
    return DeviceBatch([ds], trees, [0] * len(trees), d, nu, phi, compat=compat, mask=mask,
                       fix_nu=fix_nu, fix_phi=fix_phi, want_post=want_post, device=device,
                       stream=stream, ultrametric=ultrametric)
