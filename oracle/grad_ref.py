"""FP64 torch autograd reference of the log-likelihood (oracle; TEST
INFRASTRUCTURE ONLY).

A batched, differentiable restatement of the same generated functions as
``oracle.rv`` (``support/models/kep00-kep07.model``, ``sinusoid00.model``,
``magneticcycle00.model``, ``offset00.model``, ``jitter00.model``, the MA
recurrence of ``moav01.model``, ``acc.model``,
``support/likelihoods/00.like``) in FP64 torch, so that
``torch.autograd.grad`` gives the reference gradient the adjoint kernel is
checked against.  The Kepler equation is solved without gradient and then
differentiated through one Newton step at the solution, which yields the
implicit-function derivatives dE/dM = 1/(1 - e cos E), dE/de = sin E/(1 - e cos E).
"""
from __future__ import annotations

import numpy as np
import torch


class TorchRV:
    def __init__(self, spec, data, device='cpu'):
        self.spec = spec
        self.dev = torch.device(device)
        f64 = dict(dtype=torch.float64, device=self.dev)
        X = np.asarray(data['X'], dtype=np.float64)
        flag = np.asarray(data['Flag'])
        self.nins = int(spec['nins'])
        self.X = torch.tensor(X, **f64)
        self.Y = torch.tensor(np.asarray(data['Y'], dtype=np.float64), **f64)
        self.S2 = torch.tensor(np.asarray(data['YERR'], dtype=np.float64) ** 2, **f64)
        self.flag = torch.tensor(flag - 1, dtype=torch.long, device=self.dev)
        self.n = len(X)
        self.const = -0.5 * np.log(2 * np.pi) * self.n
        self.blocks = spec['blocks']
        blen = 0
        self.slices = []
        fixed = []
        for b in self.blocks:
            self.slices.append(slice(blen, blen + len(b['params'])))
            blen += len(b['params'])
            fixed += [p.get('fixed') for p in b['params']]
        self.n_full = blen
        self.free_idx = [i for i, f in enumerate(fixed) if f is None]
        self.fixed = {i: float(f) for i, f in enumerate(fixed) if f is not None}
        # MA sequences: per-instrument runs (documented form) or global order
        self.ma = None
        for b in self.blocks:
            if b['type'] == 'MOAV' and (b['global'] or not spec.get('moav_reference_quirk')):
                q = int(b['order'])
                if b['global']:
                    seqs = [np.arange(self.n)]
                else:
                    seqs = [np.nonzero(flag == k + 1)[0] for k in range(self.nins)]
                self.ma = (q, b['global'], seqs)

    def full(self, theta):
        B = theta.shape[0]
        cols = []
        fi = 0
        for i in range(self.n_full):
            if i in self.fixed:
                cols.append(torch.full((B,), self.fixed[i], dtype=theta.dtype, device=theta.device))
            else:
                cols.append(theta[:, fi])
                fi += 1
        return torch.stack(cols, dim=1)

    @staticmethod
    def elements(par, v):
        """(period, K, phase, tp or None, e, cos w, sin w) of one Keplerian
        block [B, 5], differentiable: the prologues of kep00-kep07.model
        (the angles of (S, C) and (As, Ac) through their cosines and sines
        directly; a 2 pi shift of the phase leaves the model unchanged)."""
        c = [v[:, i:i + 1] for i in range(5)]
        per = torch.exp(c[0]) if par in (2, 6, 7) else c[0]
        tp = None
        if par in (0, 3, 6):
            e, w = c[3], c[4]
            cw, sw = torch.cos(w), torch.sin(w)
        else:
            S, C = c[3], c[4]
            e = S * S + C * C
            r = torch.sqrt(e)
            small = e < (1e-5 if par in (2, 4) else 1e-6)
            one = torch.ones_like(e)
            cw = torch.where(small, one, C / torch.where(small, one, r))
            sw = torch.where(small, torch.zeros_like(e), S / torch.where(small, one, r))
        if par == 2:
            As, Ac = c[1], c[2]
            K = As * As + Ac * Ac
            phase = torch.atan2(As, Ac)
        else:
            K = c[1]
            phase = c[2]
        if par in (3, 4):
            tp, phase = c[2], None
        return per, K, phase, tp, e, cw, sw

    @staticmethod
    def kepler(M, e):
        # the iterations on detached values (no derivative through them, in
        # reverse or forward mode), then one Newton step with the graph:
        # exact first derivatives at the root
        Md, ed = M.detach(), e.detach()
        Mr = torch.remainder(Md + np.pi, 2 * np.pi) - np.pi
        E = Mr + 0.85 * ed * torch.sign(torch.sin(Mr))
        for _ in range(60):
            f = E - ed * torch.sin(E) - Mr
            E = E - f / (1 - ed * torch.cos(E))
        E = E + (Md - Mr)
        return E - (E - e * torch.sin(E) - M) / (1 - e * torch.cos(E))

    def loglike(self, theta):
        return torch.sum(self.terms(theta), dim=1) + self.const

    def terms(self, theta):
        """Per-epoch terms -(r_i^2 / err2_i + ln err2_i) / 2 [B, n]."""
        th = self.full(theta)
        B = th.shape[0]
        X = self.X[None, :]
        model = torch.zeros(B, self.n, dtype=th.dtype, device=th.device)
        err2 = self.S2[None, :].expand(B, -1).clone()
        resid = None
        for b, sl in zip(self.blocks, self.slices):
            v = th[:, sl]
            if b['type'] == 'Keplerian':
                per, K, phase, tp, e, cw, sw = self.elements(b['parameterisation'], v)
                M = 2 * np.pi / per * (X - tp) if tp is not None else 2 * np.pi / per * X + phase
                E = self.kepler(M, e.expand_as(M))
                cE, sE = torch.cos(E), torch.sin(E)
                D = 1 - e * cE
                q = torch.sqrt(1 - e * e)
                model = model + K * (((cE - e) * cw - q * sE * sw) / D + e * cw)
            elif b['type'] == 'Sinusoid':                     # sinusoid00.model
                P, A, phase = [v[:, i:i + 1] for i in range(3)]
                model = model + A * torch.cos(2 * np.pi / P * X + phase)
            elif b['type'] == 'MagneticCycle':                # magneticcycle00.model
                P, A1, A2, ph1, ph2 = [v[:, i:i + 1] for i in range(5)]
                model = model + A1 * torch.cos(np.pi / P * X + ph1) + A2 * torch.cos(2 * np.pi / P * X + ph2)
            elif b['type'] == 'Acceleration':
                x = X - X[:, :1]
                pv = torch.zeros_like(model)
                for j in range(v.shape[1]):
                    pv = pv * x + v[:, j:j + 1]
                model = model + pv * x
            elif b['type'] == 'Offset':
                model = model + v[:, self.flag]
            elif b['type'] == 'Jitter':
                err2 = err2 + v[:, self.flag] ** 2
            elif b['type'] == 'MOAV':
                resid = self.Y[None, :] - model
                if self.ma is not None:
                    resid = self._moav(resid, v)
        if resid is None:
            resid = self.Y[None, :] - model
        return -0.5 * (resid ** 2 / err2 + torch.log(err2))

    def _moav(self, resid, v):
        q, is_global, seqs = self.ma
        out = [None] * self.n
        cols = list(resid.unbind(1))
        for k, idx in enumerate(seqs):
            base = 0 if is_global else 2 * q * k
            t = self.X[idx]
            prev = []
            for ii, i in enumerate(idx):
                x = cols[i]
                for c in range(q):
                    if ii > c:
                        dt = torch.abs(t[ii] - t[ii - 1 - c])
                        a = v[:, base + 2 * c] * torch.exp(-dt / v[:, base + 2 * c + 1])
                        x = x - a * prev[ii - 1 - c]
                prev.append(x)
                out[i] = x
        return torch.stack(out, dim=1)

    def condition(self, theta, chunk=100):
        """sum_i |d term_i / d theta_j| [B, ndim]: the size of the summands of
        each gradient component (forward-mode derivatives of the per-epoch
        terms); a component computed from rounded terms is only defined to
        the terms' rounding times this."""
        th = torch.as_tensor(theta, dtype=torch.float64, device=self.dev)
        out = torch.zeros_like(th)
        for b0 in range(0, th.shape[0], chunk):
            x = th[b0:b0 + chunk]
            for j in range(x.shape[1]):
                t = torch.zeros_like(x)
                t[:, j] = 1.0
                _, d = torch.func.jvp(self.terms, (x,), (t,))
                out[b0:b0 + chunk, j] = d.abs().sum(1)
        return out.cpu().numpy()

    def grad(self, theta):
        th = torch.as_tensor(theta, dtype=torch.float64, device=self.dev).clone().requires_grad_(True)
        ll = self.loglike(th)
        g, = torch.autograd.grad(ll.sum(), th)
        return ll.detach().cpu().numpy(), g.detach().cpu().numpy()
