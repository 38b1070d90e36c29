"""Mirror of fast_em/laml.py: EMOptimizer (196-276) and
optimize_parameters_expectation_maximization (112-194) on the GB300 engine.

The M-step maximises the same objective (M_step_loss_fn, laml.py:62-78) to
its stationary point by coordinate ascent (closed-form phi, per-branch and nu
Newton solves) instead of 100 optax L-BFGS steps; the EM loop, stopping rule
(relative change < 1e-5), NaN guard and return convention (parameters from
before the last M-step on convergence) are the reference's.
"""
from __future__ import annotations

import numpy as np

from ..engine import MSTEP_ROUNDS, DeviceBatch
from ._adapt import as_numpy, dataset_from_dense, tree_from_arrays, tree_from_networkx

M_STEP_DESCENT_STEPS = 100      # laml.py:45 (kept for reference; see module doc)
EM_STOPPING_CRITERION = 1e-5    # laml.py:46
EPS = 1e-6


def _run(ds, tr, d, nu, phi, mask, fix_nu, fix_phi, rounds=MSTEP_ROUNDS):
    nu = min(max(float(nu), EPS), 1 - EPS)
    phi = min(max(float(phi), EPS), 1 - EPS)
    d = np.maximum(as_numpy(d, np.float64), EPS)
    b = DeviceBatch([ds], [tr], [0], [d], [nu], [phi], compat=True,
                    mask=None if mask is None else [as_numpy(mask).astype(bool)],
                    fix_nu=fix_nu, fix_phi=fix_phi)
    return b.run_em(rounds=rounds, rel_tol=EM_STOPPING_CRITERION)[0]


def optimize_parameters_expectation_maximization(leaves, internal_postorder,
                                                 internal_postorder_children, parent_sibling,
                                                 level_order, inside_log_likelihoods,
                                                 model_parameters, model_parameters_mask,
                                                 character_matrix, branch_lengths, branch_mask,
                                                 mutation_priors, root, verbose=False):
    """Returns (log-likelihood, branch lengths, (nu, phi), EM iterations) as
    laml.py:194 does (its first value is named current_nllh there but holds
    the log-likelihood)."""
    d = as_numpy(branch_lengths, np.float64)
    tr = tree_from_arrays(len(d), leaves, internal_postorder, internal_postorder_children)
    ds = dataset_from_dense(mutation_priors, character_matrix)
    mp = as_numpy(model_parameters, np.float64)
    pm = as_numpy(model_parameters_mask, np.float64)
    r = _run(ds, tr, d, mp[0], mp[1], branch_mask, pm[0] == 0, pm[1] == 0)
    return r.llh, r.branch_lengths, (r.nu, r.phi), r.iterations


class EMOptimizer:
    """fast_em/laml.py:196-276.  ``mutation_priors`` (K, M) and
    ``character_matrix`` (n, K) as built by build_phylogeny; their device
    encoding is made once and reused by every ``optimize`` call."""

    def __init__(self, mutation_priors, character_matrix, verbose=False):
        self.mutation_priors = as_numpy(mutation_priors, np.float32)
        self.character_matrix = as_numpy(character_matrix).astype(np.int32)
        self.num_leaves = self.character_matrix.shape[0]
        self.alphabet_size = self.mutation_priors.shape[1]
        self.num_characters = self.character_matrix.shape[1]
        self.verbose = verbose
        self._ds = dataset_from_dense(self.mutation_priors, self.character_matrix)

    def optimize(self, tree, branch_lengths, nu, phi, branch_mask, fixed_nu=False,
                 fixed_phi=False):
        tr = tree_from_networkx(tree)
        if tr.num_leaves != self.num_leaves:
            raise ValueError("tree and character matrix have different numbers of leaves")
        r = _run(self._ds, tr, branch_lengths, nu, phi, branch_mask, bool(fixed_nu),
                 bool(fixed_phi))
        return {"nllh": -r.llh, "branch_lengths": r.branch_lengths, "nu": r.nu, "phi": r.phi,
                "em_iterations": r.iterations}
