"""Differentiable PMM log-likelihood: a torch.autograd.Function whose
backward is the hand-written adjoint of the inside pass.

forward: branch terms -> inside pass -> per-tree log-likelihood (FP64 sum).
backward: outside pass with the true root counts -> expected transition counts
-> d logL / d(branch lengths, nu, phi) (``DeviceBatch.gradient``, the
laml_gradient kernel).  By Fisher's identity this is the exact gradient of
log L: the gradient of the expected complete-data log-likelihood (the
objective of fast_em/laml.py:62-78 with true root counts) at the current
parameters.

``recompute=True`` re-runs the inside pass in backward instead of relying on
the partials the forward left in the batch's buffers (use it when other work
reuses the batch between forward and backward).
"""
from __future__ import annotations

import torch

from .engine import DeviceBatch


class PMMLogLikelihood(torch.autograd.Function):
    @staticmethod
    def forward(ctx, d, nu, phi, batch: DeviceBatch, recompute: bool = False):
        batch.set_params(d.detach(), nu.detach(), phi.detach())
        batch.branch_terms()
        batch.inside(update_em=False)
        llh = batch.work["tr_llh"].clone()
        ctx.batch = batch
        ctx.recompute = recompute
        ctx.save_for_backward(d, nu, phi)
        return llh

    @staticmethod
    def backward(ctx, g):
        b: DeviceBatch = ctx.batch
        d, nu, phi = ctx.saved_tensors
        if ctx.recompute:
            b.set_params(d.detach(), nu.detach(), phi.detach())
            b.branch_terms()
            b.inside(update_em=False)
        b.outside(true_root=True)
        gd, gnu, gphi = b.gradient()
        node_tree = b.v["nd_tree"].long()
        g = g.to(torch.float64)
        return (g[node_tree] * gd).to(d.dtype), (g * gnu).to(nu.dtype), (g * gphi).to(phi.dtype), \
            None, None


def log_likelihood(d: torch.Tensor, nu: torch.Tensor, phi: torch.Tensor, batch: DeviceBatch,
                   recompute: bool = False) -> torch.Tensor:
    """Per-tree log-likelihood [T], differentiable in d [n_nodes], nu [T],
    phi [T] (float64 CUDA tensors)."""
    return PMMLogLikelihood.apply(d, nu, phi, batch, recompute)
