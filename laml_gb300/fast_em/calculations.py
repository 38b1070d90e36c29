"""Mirror of fast_em/calculations.py's public entry points on the GB300 engine.

``compute_log_likelihood`` (calculations.py:456-504) and ``compute_E_step``
(calculations.py:506-577) take the same eleven positional arguments (numpy
or torch arrays); ``inside_log_likelihoods`` is accepted and ignored (the
engine owns its partial buffers).  Values follow the reference's fastEM
semantics (EPS floors, observed-state priors, root E-step row from node
N-1); arithmetic is FP32 with FP64 site sums.
"""
from __future__ import annotations

import numpy as np

from ..engine import DeviceBatch
from ._adapt import as_numpy, dataset_from_dense, tree_from_arrays

EPS = 1e-6


def _batch(branch_lengths, mutation_priors, leaves, internal_postorder,
           internal_postorder_children, model_parameters, character_matrix):
    d = as_numpy(branch_lengths, np.float64)
    tr = tree_from_arrays(len(d), leaves, internal_postorder, internal_postorder_children)
    ds = dataset_from_dense(mutation_priors, character_matrix)
    nu, phi = (float(x) for x in as_numpy(model_parameters, np.float64)[:2])
    return DeviceBatch([ds], [tr], [0], [d], [nu], [phi], compat=True)


def compute_log_likelihood(branch_lengths, mutation_priors, leaves, internal_postorder,
                           internal_postorder_children, parent_sibling, level_order,
                           inside_log_likelihoods, model_parameters, character_matrix, root):
    b = _batch(branch_lengths, mutation_priors, leaves, internal_postorder,
               internal_postorder_children, model_parameters, character_matrix)
    return float(b.log_likelihood()[0])


def compute_E_step(branch_lengths, mutation_priors, leaves, internal_postorder,
                   internal_postorder_children, parent_sibling, level_order,
                   inside_log_likelihoods, model_parameters, character_matrix, root):
    """(log-likelihood, expected counts (N, 6) = [C00, C0a, C0s, Caa, Cas, Css]
    summed over sites, per-leaf silenced responsibilities (n,))."""
    b = _batch(branch_lengths, mutation_priors, leaves, internal_postorder,
               internal_postorder_children, model_parameters, character_matrix)
    b.e_step()
    cnt, lr = b.counts_from_partials()
    llh = float(b.work["tr_llh"].cpu().numpy()[0])
    n = len(as_numpy(leaves))
    return llh, cnt, lr[0][:n]
