"""``torch.autograd.Function`` over the log-posterior kernels.

Forward runs the log-posterior kernel (mixed or FP64); backward runs the
hand-written adjoint kernel (``emp_logpost_grad``), which recomputes the
eccentric anomaly instead of storing it.  Walkers outside the prior support
have log-posterior -inf and a zero gradient.
"""
from __future__ import annotations

import torch

from . import _native as N


class EmpLogPosterior(torch.autograd.Function):
    @staticmethod
    def forward(fctx, theta, context, precision=N.EMP_PREC_MIXED, include_prior=True):
        th = theta.detach().contiguous()
        ll, lp = context.logpost(th, precision=precision)
        fctx.context = context
        fctx.include_prior = include_prior
        fctx.save_for_backward(th)
        return ll + lp if include_prior else ll

    @staticmethod
    def backward(fctx, gout):
        th, = fctx.saved_tensors
        _, lp, gl, gp = fctx.context.logpost_grad(th)
        g = gl + gp if fctx.include_prior else gl
        g = torch.where(torch.isfinite(lp)[:, None], g, torch.zeros_like(g))
        return gout[:, None] * g, None, None, None


def log_posterior(theta, context, precision=N.EMP_PREC_MIXED, include_prior=True):
    """logL + logprior (or logL) of theta [B, ndim], differentiable in theta."""
    return EmpLogPosterior.apply(theta, context, precision, include_prior)
