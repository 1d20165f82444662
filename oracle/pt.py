"""numpy parallel-tempering engine (oracle; TEST INFRASTRUCTURE ONLY).

Restates the sampler EMPEROR drives through ``reddemcee.PTSampler``
(``src/astroemperor/emp.py:576-593``; ``support/endit_reddemcee.scr:3``).
reddemcee (``requirements.txt:248`` pins 0.8.5) and emcee 3.1.6
(``requirements.txt:54-55``) are not vendored in the reference and are not
installed here, so their published algorithms are restated:

* stretch move -- Goodman & Weare (2010), as emcee 3's ``StretchMove`` on a
  two-way split of each temperature's ensemble: for walker j of half h a
  partner k is drawn from the other half, ``z = ((a-1) u + 1)^2 / a``,
  ``Y = X_k - (X_k - X_j) z``, accepted when
  ``(ndim-1) ln z + logP(Y) - logP(X_j) > ln u'``, with the tempered
  ``logP = beta logL + logprior``;
* swaps -- adjacent pairs from the hottest down; walker j of temperature i
  against walker pi(j) of temperature i-1, accepted when
  ``(beta_{i-1} - beta_i)(logL_i - logL_{i-1}) > ln u``;
* ladder adaptation -- Vousden, Farr & Mandel (2016):
  ``dT_k <- dT_k exp(kappa (A_k - A_{k+1}))``,
  ``kappa = adapt_tau / (t + adapt_tau) / adapt_nu``, ends fixed.

The engine can draw from :mod:`oracle.philox` with the device's counter
layout (``rng='philox'``), which makes its chains identical to the device
sampler's, or from numpy (``rng='numpy'``) for independent-stream
Monte-Carlo comparisons.
"""
from __future__ import annotations

import math

import numpy as np

from . import philox as ph


def perm_units(W):
    return np.array([m for m in range(1, max(W, 2)) if math.gcd(m, W) == 1] or [1], dtype=np.int64)


class OraclePT:
    def __init__(self, logpost, ntemps, nwalkers, ndim, betas, a=2.0, adapt=True,
                 adapt_tau=1000.0, adapt_nu=1.0, rng='philox', seed=0):
        """``logpost(theta[B, D]) -> (logl[B], logprior[B])``."""
        self.logpost = logpost
        self.T, self.W, self.D = int(ntemps), int(nwalkers), int(ndim)
        self.betas = np.array(betas, dtype=np.float64)
        self.a = float(a)
        self.adapt = bool(adapt)
        self.adapt_tau, self.adapt_nu = float(adapt_tau), float(adapt_nu)
        self.rng_kind = rng
        self.seed = int(seed)
        self.np_rng = np.random.default_rng(seed)
        self.units = perm_units(self.W)
        self.steps = 0
        self.sweeps = 0
        self.accepted = np.zeros((self.T, self.W), dtype=np.int64)
        self.swaps_accepted = np.zeros(self.T, dtype=np.int64)
        self.chain, self.log_like, self.log_prob = [], [], []
        self.beta_hist, self.tsw_hist, self.smd_hist = [], [], []

    def set_positions(self, p0):
        p0 = np.asarray(p0, dtype=np.float64)
        self.theta = p0.reshape(self.T * self.W, self.D).copy()
        self.members = np.arange(self.T * self.W).reshape(self.T, self.W)
        self.logl, self.logprior = self.logpost(self.theta)
        self.logl = np.asarray(self.logl, dtype=np.float64).copy()
        self.logprior = np.asarray(self.logprior, dtype=np.float64).copy()

    def _logP(self, ll, lp, beta):
        return np.where(lp > -np.inf, beta * ll + lp, -np.inf)

    def stretch_half(self, half, step_in_sweep):
        T, W, D = self.T, self.W, self.D
        Wh = W // 2
        t = np.repeat(np.arange(T), Wh)
        jj = np.tile(np.arange(Wh), T)
        j = 2 * jj + half
        idx = t * W + j
        if self.rng_kind == 'philox':
            it = self.steps + step_in_sweep
            x0, x1, x2, x3 = ph.draw(self.seed, idx.astype(np.uint32), it, ph.STRETCH0 + half)
            kk = ph.mulhi(x2, Wh)
            uz = ph.u53(x0, x1)
            logu = np.log(ph.u32u(x3))
        else:
            kk = self.np_rng.integers(0, Wh, size=len(idx))
            uz = self.np_rng.random(len(idx))
            logu = np.log(self.np_rng.random(len(idx)))
        k = 2 * kk + (1 - half)
        sj = self.members[t, j]
        sk = self.members[t, k]
        zz = (self.a - 1.0) * uz + 1.0
        z = zz * zz / self.a
        ck = self.theta[sk]
        q = ck - (ck - self.theta[sj]) * z[:, None]
        nll, nlp = self.logpost(q)
        nll = np.asarray(nll, dtype=np.float64)
        nlp = np.asarray(nlp, dtype=np.float64)
        beta = self.betas[t]
        cur = self._logP(self.logl[sj], self.logprior[sj], beta)
        new = self._logP(nll, nlp, beta)
        with np.errstate(invalid='ignore'):
            lnpdiff = ((D - 1.0) * np.log(z) + new) - cur
            acc = (nlp > -np.inf) & (lnpdiff > logu)
        self.theta[sj[acc]] = q[acc]
        self.logl[sj[acc]] = nll[acc]
        self.logprior[sj[acc]] = nlp[acc]
        self.accepted[t[acc], j[acc]] += 1
        return acc

    def swap_and_adapt(self):
        T, W, D = self.T, self.W, self.D
        betas_used = self.betas.copy()
        ratio = np.zeros(max(T - 1, 0))
        smd = np.zeros(max(T - 1, 0))
        for i in range(T - 1, 0, -1):
            if self.rng_kind == 'philox':
                x0, x1, _, _ = ph.draw(self.seed, np.uint32(i), self.sweeps, ph.SWAP_PERM)
                m = int(self.units[int(x0) % len(self.units)])
                b = int(x1) % W
                j = np.arange(W)
                jp = (m * j + b) % W
                a0, _, _, _ = ph.draw(self.seed, (i * W + j).astype(np.uint32), self.sweeps, ph.SWAP_ACC)
                logu = np.log(ph.u32u(a0))
            else:
                j = np.arange(W)
                jp = self.np_rng.permutation(W)
                logu = np.log(self.np_rng.random(W))
            dbeta = self.betas[i - 1] - self.betas[i]
            sa = self.members[i, j].copy()
            sb = self.members[i - 1, jp].copy()
            with np.errstate(invalid='ignore'):
                pacc = dbeta * (self.logl[sa] - self.logl[sb])
                acc = logu < pacc
            self.members[i, j[acc]] = sb[acc]
            self.members[i - 1, jp[acc]] = sa[acc]
            c = int(acc.sum())
            ratio[i - 1] = c / W
            if c:
                dist = np.sqrt(np.sum((self.theta[sa[acc]] - self.theta[sb[acc]]) ** 2, axis=1))
                smd[i - 1] = dist.sum() / c
            self.swaps_accepted[i] += c
        self.beta_hist.append(betas_used)
        self.tsw_hist.append(ratio)
        self.smd_hist.append(smd)
        if self.adapt and T > 2:
            kappa = self.adapt_tau / (self.sweeps + self.adapt_tau) / self.adapt_nu
            invb = 1.0 / self.betas[:-1]
            cum = invb[0]
            for k in range(T - 2):
                cum += (invb[k + 1] - invb[k]) * np.exp(kappa * (ratio[k] - ratio[k + 1]))
                self.betas[k + 1] = 1.0 / cum
        return betas_used

    def sweep(self, nsteps=1):
        for s in range(nsteps):
            self.stretch_half(0, s)
            self.stretch_half(1, s)
        betas_used = self.swap_and_adapt()
        self.steps += nsteps
        self.sweeps += 1
        m = self.members.reshape(-1)
        self.chain.append(self.theta[m].reshape(self.T, self.W, self.D).copy())
        ll = self.logl[m].reshape(self.T, self.W)
        lp = self.logprior[m].reshape(self.T, self.W)
        self.log_like.append(ll.copy())
        self.log_prob.append(self._logP(ll, lp, betas_used[:, None]))

    def run(self, nsweeps, nsteps=1):
        for _ in range(int(nsweeps)):
            self.sweep(nsteps)
        return self
