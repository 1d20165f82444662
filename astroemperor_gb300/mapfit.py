"""Multistart MAP search driven by the adjoint kernel, for walker initialisation.

Each start runs L-BFGS (two-loop recursion, memory ``m``, Armijo
backtracking) on -log posterior in an unconstrained coordinate u with
theta = lo + (hi - lo) * sigmoid(u) per free parameter, so every iterate
stays inside the prior limits.  All starts advance together: one gradient
kernel launch per line-search trial evaluates every start.  Points outside
the derived supports (e.g. S^2 + C^2 > 1) have -log posterior = +inf and
are rejected by the line search.  The bookkeeping of the recursion is eager
torch on [starts, ndim] tensors (a few dozen small elementwise kernels per
iteration); it is off the sampling path, and the gradient kernel dominates
the time.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _native as N


def _to_theta(u, lo, span):
    s = torch.sigmoid(u)
    return lo + span * s, span * s * (1 - s)


def _objective(ctx, u, lo, span):
    th, jac = _to_theta(u, lo, span)
    ll, lp, gl, gp = ctx.logpost_grad(th)
    f = -(ll + lp)
    g = -(gl + gp) * jac
    bad = ~torch.isfinite(f)
    f = torch.where(bad, torch.full_like(f, math.inf), f)
    g = torch.where(bad[:, None], torch.zeros_like(g), g)
    return f, g


def multistart_map(ctx, model, theta0: torch.Tensor, iters=300, m=8, tol=1e-12, max_ls=25, gtol=1e-5):
    """L-BFGS from every row of theta0 [S, D] (inside the limits).

    A start stops when its objective changes by less than ``tol`` relative,
    when no step along the search direction decreases it (the line search
    fails: converged to the precision of the objective), or when the largest
    component of its gradient in the unconstrained coordinates falls below
    ``gtol``.  Returns dict with theta [S, D], logp [S] (log posterior),
    iterations, evaluations (gradient-kernel launches, each over all starts)
    and converged [S] (stopped before ``iters``).
    """
    dev = theta0.device
    lim = torch.as_tensor(model.limits_free(), dtype=torch.float64, device=dev)
    lo, span = lim[:, 0], lim[:, 1] - lim[:, 0]
    p = ((theta0 - lo) / span).clamp(1e-9, 1 - 1e-9)
    u = torch.log(p) - torch.log1p(-p)
    f, g = _objective(ctx, u, lo, span)
    evals = 1
    S, D = u.shape
    sh = torch.zeros(m, S, D, dtype=torch.float64, device=dev)
    yh = torch.zeros_like(sh)
    rho = torch.zeros(m, S, dtype=torch.float64, device=dev)
    k = 0
    active = torch.isfinite(f)
    for it in range(iters):
        # two-loop recursion for d = -H g
        q = g.clone()
        alpha = torch.zeros(m, S, dtype=torch.float64, device=dev)
        nh = min(k, m)
        for i in range(nh):
            j = (k - 1 - i) % m
            alpha[j] = rho[j] * (sh[j] * q).sum(1)
            q = q - alpha[j][:, None] * yh[j]
        if nh > 0:
            j = (k - 1) % m
            yy = (yh[j] * yh[j]).sum(1)
            gamma = torch.where(yy > 0, (sh[j] * yh[j]).sum(1) / yy, torch.ones_like(yy))
            r = gamma[:, None] * q
        else:
            r = q / g.norm(dim=1, keepdim=True).clamp_min(1.0)
        for i in range(nh - 1, -1, -1):
            j = (k - 1 - i) % m
            beta = rho[j] * (yh[j] * r).sum(1)
            r = r + (alpha[j] - beta)[:, None] * sh[j]
        d = -r
        gd = (g * d).sum(1)
        # not a descent direction: fall back to steepest descent
        bad = ~(gd < 0)
        d = torch.where(bad[:, None], -g, d)
        gd = torch.where(bad, -(g * g).sum(1), gd)
        step = torch.ones(S, dtype=torch.float64, device=dev)
        done = ~active
        u_new, f_new, g_new = u.clone(), f.clone(), g.clone()
        for _ in range(max_ls):
            trial = u + step[:, None] * d
            ft, gt = _objective(ctx, trial, lo, span)
            evals += 1
            ok = (~done) & (ft <= f + 1e-4 * step * gd)
            u_new = torch.where(ok[:, None], trial, u_new)
            f_new = torch.where(ok, ft, f_new)
            g_new = torch.where(ok[:, None], gt, g_new)
            done = done | ok
            if bool(done.all()):
                break
            step = torch.where(done, step, 0.5 * step)
        moved = done & active
        s_vec = u_new - u
        y_vec = g_new - g
        sy = (s_vec * y_vec).sum(1)
        upd = moved & (sy > 1e-12)
        j = k % m
        sh[j] = torch.where(upd[:, None], s_vec, sh[j])
        yh[j] = torch.where(upd[:, None], y_vec, yh[j])
        rho[j] = torch.where(upd, 1.0 / sy.clamp_min(1e-300), rho[j])
        k += 1
        rel = (f - f_new).abs() / f_new.abs().clamp_min(1.0)
        u, f, g = u_new, f_new, g_new
        small_g = g.abs().amax(dim=1) < gtol
        active = active & ~(rel < tol) & ~small_g & torch.isfinite(f)
        if not bool(active.any()):
            break
    th, _ = _to_theta(u, lo, span)
    return {'theta': th, 'logp': -f, 'iterations': it + 1, 'evaluations': evals,
            'converged': ~active}


def walkers_around(best: torch.Tensor, model, ntemps, nwalkers, scale=1e-4, seed=0):
    """Walkers [T, W, D] scattered around a MAP point, inside the limits."""
    lim = model.limits_free()
    rng = np.random.default_rng(seed)
    b = best.detach().cpu().numpy()
    p = b + scale * (lim[:, 1] - lim[:, 0]) * rng.normal(size=(ntemps, nwalkers, len(b)))
    return np.clip(p, lim[:, 0], lim[:, 1])
