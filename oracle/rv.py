"""FP64 numpy restatement of EMPEROR's generated RV log-posterior (oracle).

TEST INFRASTRUCTURE ONLY -- never imported by the product package.

Every function below restates one piece of the reference and cites it
(paths relative to the reference project root):

* data preprocessing ......... ``src/astroemperor/qol_utils.py:61-100, 192-198``
* data prologue / masks ...... ``src/astroemperor/emp_model.py:406-433``
* model assembly order ....... ``src/astroemperor/emp_model.py:706-781``
* Keplerian parameterisations  ``src/astroemperor/support/models/kep00..kep07.model``
* offset / jitter ............ ``support/models/offset00.model:3``, ``jitter00.model:3``
* moving average ............. ``support/models/moav00.model`` (per instrument),
                               ``support/models/moav01.model`` (global)
* acceleration ............... ``support/models/acc.model:2``
* Gaussian likelihood ........ ``support/likelihoods/00.like:1-5``; with
                               astrometry ``a00.like`` (``oracle/am.py``)
* priors ..................... ``support/priors/{Uniform,Normal,Jeffreys,Beta,Fixed,Isotropic}.prior``
                               with normalisers from ``emp_model.py:82-120``
* prior writer (my_prior) .... ``src/astroemperor/emp.py:182-254``

The Kepler equation is solved by this module's own FP64 Halley iteration
(the reference calls the third-party ``kepler.py`` 0.0.7 ``kepler.solve``,
which is not available here); any converged solver agrees to ~1e-15 rad.

The model is described by a plain "model spec" dict (see
``astroemperor_gb300.model.ReddModel.spec``)::

    {'nins': n,
     'moav_reference_quirk': bool,
     'blocks': [
        {'type': 'Keplerian', 'parameterisation': p,
         'params': [{'name', 'prior', 'limits', 'prargs', 'fixed'} x 5],
         'additional': [{'name', 'prior', 'limits', 'prargs', 'has_prior'}]},
        {'type': 'Acceleration', 'params': [...]},
        {'type': 'Offset', 'params': [... n]},
        {'type': 'Jitter', 'params': [... n]},
        {'type': 'MOAV', 'order': q, 'global': bool, 'params': [...]}]}
"""
from __future__ import annotations

import math
import os

import numpy as np
from scipy.stats import beta as _betapdf
from scipy.stats import norm as _norm

TWO_PI = 2.0 * np.pi


# --------------------------------------------------------------------------
# data preprocessing  (qol_utils.py:61-100, 192-198)
# --------------------------------------------------------------------------
def read_vels_folder(folder):
    """List of per-instrument (BJD, RV, eRV) arrays from ``*.vels`` files.

    ``DataWrapper.activate`` reads the instrument files in ``sorted(os.listdir)``
    order and ``mk_RV`` loads each with ``np.loadtxt`` (qol_utils.py:47-100).
    """
    names = [fn for fn in sorted(os.listdir(folder)) if fn != '.DS_Store']
    out = []
    for fn in names:
        d = np.loadtxt(os.path.join(folder, fn), ndmin=2)
        out.append(d[:, :3].copy())
    return out, names


def preprocess(instruments):
    """Restates ``DataWrapper.mk_RV`` + ``get_data__``.

    * each instrument's RV has its own mean subtracted when |mean| > 1e-6
      (qol_utils.py:84-85);
    * ``Flag`` = 1-based instrument index (qol_utils.py:95);
    * rows are concatenated and sorted by BJD, and ``common_t = min(BJD)``
      is subtracted (qol_utils.py:192-198).  A stable sort is used; the
      reference's pandas quicksort leaves the order of exactly tied BJD
      values unspecified.
    """
    bjd, rv, erv, flag = [], [], [], []
    for k, d in enumerate(instruments):
        d = np.asarray(d, dtype=np.float64)
        r = d[:, 1].copy()
        m = r.mean()
        if abs(m) > 1e-6:
            r = r - m
        bjd.append(d[:, 0])
        rv.append(r)
        erv.append(d[:, 2])
        flag.append(np.full(len(d), k + 1, dtype=np.int64))
    bjd = np.concatenate(bjd)
    rv = np.concatenate(rv)
    erv = np.concatenate(erv)
    flag = np.concatenate(flag)
    order = np.argsort(bjd, kind='mergesort')
    bjd, rv, erv, flag = bjd[order], rv[order], erv[order], flag[order]
    common_t = bjd.min()
    return {'X': bjd - common_t, 'Y': rv, 'YERR': erv, 'Flag': flag,
            'common_t': common_t, 'nins': len(instruments)}


# --------------------------------------------------------------------------
# Kepler equation (kepler.py 0.0.7 ``kepler.solve(M, e)`` call sites:
# support/models/kep00.model:6, kep01.model:13)
# --------------------------------------------------------------------------
def kepler_solve(M, e, tol=1e-15, maxiter=60):
    """Eccentric anomaly E with M = E - e sin E, for 0 <= e < 1 (FP64).

    M is reduced to [-pi, pi); the start is Danby's E0 = M + 0.85 e sign(sin M),
    from which Halley's iteration converges for every (M, e) with e < 1.
    The returned E lies in [-pi, pi]; the reference only uses tan(E/2), which
    has period 2 pi, so the branch does not matter.
    """
    M = np.asarray(M, dtype=np.float64)
    e = np.broadcast_to(np.asarray(e, dtype=np.float64), M.shape)
    Mr = np.remainder(M + np.pi, TWO_PI) - np.pi
    E = Mr + 0.85 * e * np.sign(np.sin(Mr))
    for _ in range(maxiter):
        s, c = np.sin(E), np.cos(E)
        f = E - e * s - Mr
        f1 = 1.0 - e * c
        f2 = e * s
        d1 = -f / f1
        d = -f / (f1 + 0.5 * d1 * f2)
        E = E + d
        if np.all(np.abs(d) <= tol):
            break
    return E


# --------------------------------------------------------------------------
# prior normalisers (emp_model.py:82-120) and prior functions
# (support/priors/*.prior)
# --------------------------------------------------------------------------
def check_prargs(prior, limits, prargs):
    """Restates ``Parameter_Block._check_prargs`` (emp_model.py:82-98)."""
    if prior == 'Uniform':
        low, high = limits
        return np.log(1 / (high - low))
    if prior == 'Normal':
        low, high = limits
        mu, s = prargs[0], prargs[1]
        a, b = (low - mu) / s, (high - mu) / s
        logZ = np.log(_norm.cdf(b) - _norm.cdf(a))
        return [mu, s, logZ]
    if prior == 'Isotropic':                                   # emp_model.py:96-99
        low, high = limits
        return np.log(0.5 * (np.cos(low) - np.cos(high)))
    return prargs


def prior_Uniform(x, limits, args):          # support/priors/Uniform.prior:1-5
    logZ = args
    if limits[0] <= x <= limits[1]:
        return logZ
    return -np.inf


def prior_Normal(x, limits, args):           # support/priors/Normal.prior:1-9
    low, high = limits
    mu, s, logZ = args[0], args[1], args[2]
    if low <= x <= high:
        return -0.5 * ((x - mu) / s) ** 2 - np.log(s * np.sqrt(2 * np.pi)) - logZ
    return -np.inf


def prior_Jeffreys(x, limits, args):         # support/priors/Jeffreys.prior:1-6
    low, high = limits
    if low <= x <= high:
        return np.log(1 / (high - low))
    return -np.inf


def prior_Beta(x, limits, args):             # support/priors/Beta.prior:1-6
    if limits[0] <= x <= limits[1]:
        a, b = args[0], args[1]
        return np.log(_betapdf.pdf(x, a, b))
    return -np.inf


def prior_Fixed(x, limits, args):            # support/priors/Fixed.prior:1-2
    return 0.


def prior_Isotropic(x, limits, args):        # support/priors/Isotropic.prior:1-5
    logZ = args
    if limits[0] <= x <= limits[1]:
        return np.log(0.5 * np.sin(x)) - logZ
    return -np.inf


PRIORS = {'Uniform': prior_Uniform, 'Normal': prior_Normal,
          'Jeffreys': prior_Jeffreys, 'Beta': prior_Beta, 'Fixed': prior_Fixed,
          'Isotropic': prior_Isotropic}


def cps(pers, amps, eccs, starmass):
    """math_utils.py:31-61: semi-major axes (AU, Kepler's third law without
    the planet mass) and minimum masses (M_Jup) from P [d], K [m/s], e."""
    G, M_sun, AU, day = 6.6743e-11, 1.98847e30, 1.495978707e11, 86400.0
    P = np.asarray(pers, dtype=float) * day
    K = np.asarray(amps, dtype=float)
    e = np.asarray(eccs, dtype=float)
    a_m = (G * (starmass * M_sun) * P ** 2 / (4.0 * np.pi ** 2)) ** (1.0 / 3.0)
    sma = a_m / AU
    minmass = (K / 28.4329) * np.sqrt(1.0 - e ** 2) * np.sqrt(starmass * sma)
    return sma, minmass


def prior_Hill(x, limits, args):
    """support/priors/Hill.prior: 0 when every adjacent pair ordered by
    semi-major axis passes LHS > RHS, else -inf.  As in the reference, gamma
    keeps the input order while the axes and masses are sorted."""
    kplanets, starmass = args[0], args[1]
    periods, amps, eccs = x
    with np.errstate(invalid='ignore', divide='ignore'):
        gamma = np.sqrt(1 - eccs)
        sma, minmass = cps(periods, amps, eccs, starmass)
        orden = np.argsort(sma)
        sma, minmass = sma[orden], minmass[orden]
        M = starmass * 1047.56 + np.sum(minmass)
        mu = minmass / M
        for k in range(int(kplanets) - 1):
            alpha = mu[k] + mu[k + 1]
            delta = np.sqrt(sma[k + 1] / sma[k])
            LHS = alpha ** -3 * (mu[k] + (mu[k + 1] / (delta ** 2))) * \
                (mu[k] * gamma[k] + mu[k + 1] * gamma[k + 1] * delta) ** 2
            RHS = 1 + (3. / alpha) ** (4. / 3) * (mu[k] * mu[k + 1])
            if not LHS > RHS:
                return -np.inf
    return 0.


def hill_x(par, theta, b_len, kplanets):
    """support/PAE/0<par>.pae: (periods, amps, eccs) of the first kplanets
    Keplerian blocks, read from the full theta with stride b_len."""
    s = lambda i: theta[slice(i, b_len * kplanets, b_len)]
    if par in (0, 3):
        return np.array([s(0), s(1), s(3)])
    if par in (1, 4):
        return np.array([s(0), s(1), s(3) ** 2 + s(4) ** 2])
    if par == 2:
        return np.array([np.exp(s(0)), s(1) ** 2 + s(2) ** 2, s(3) ** 2 + s(4) ** 2])
    if par == 6:
        return np.array([np.exp(s(0)), s(1), s(3)])
    raise ValueError(f'no PAE script for parameterisation {par}')


# --------------------------------------------------------------------------
# the per-theta functions
# --------------------------------------------------------------------------
def kepler_rv(X, per, A, phase, ecc, w):
    """One Keplerian RV term, exactly as written in kep00/kep01.model."""
    freq = 2. * np.pi / per                                   # kep01.model:11
    M = freq * X + phase                                      # kep01.model:12
    E = kepler_solve(M, np.repeat(ecc, len(M)))               # kep01.model:13
    f = (np.arctan(((1. + ecc) ** 0.5 / (1. - ecc) ** 0.5) * np.tan(E / 2.)) * 2.)
    return A * (np.cos(f + w) + ecc * np.cos(w))              # kep01.model:15


def kepler_elements(par, v):
    """(per, A, phase_or_None, tp_or_None, ecc, w) from one 5-vector.

    Restates the prologues of support/models/kep00..kep07.model.
    """
    if par == 0:                                              # kep00.model:2
        per, A, phase, ecc, w = v
        return per, A, phase, None, ecc, w
    if par in (1, 7):                                         # kep01.model:1-9, kep07.model:2-11
        P, A, phase, S, C = v
        per = np.exp(P) if par == 7 else P
        ecc = S ** 2 + C ** 2
        if ecc < 1e-6:
            w = 0
        else:
            w = np.arccos(C / (ecc ** 0.5))
            if S < 0:
                w = 2 * np.pi - w
        return per, A, phase, None, ecc, w
    if par == 2:                                              # kep02.model:1-16
        P, As, Ac, S, C = v
        per = np.exp(P)
        A = As ** 2 + Ac ** 2
        ecc = S ** 2 + C ** 2
        if ecc < 1e-5:
            w = 0
        else:
            w = np.arccos(C / (ecc ** 0.5))
            if S < 0:
                w = 2 * np.pi - np.arccos(C / (ecc ** 0.5))
        phase = np.arccos(Ac / (A ** 0.5))
        if As < 0:
            phase = 2 * np.pi - np.arccos(Ac / (A ** 0.5))
        return per, A, phase, None, ecc, w
    if par == 3:                                              # kep03.model:1
        per, A, tp, ecc, w = v
        return per, A, None, tp, ecc, w
    if par == 4:                                              # kep04.model:1-9
        per, A, tp, S, C = v
        ecc = S ** 2 + C ** 2
        if ecc < 1e-5:
            w = 0
        else:
            w = np.arccos(C / (ecc ** 0.5))
            if S < 0:
                w = 2 * np.pi - np.arccos(C / (ecc ** 0.5))
        return per, A, None, tp, ecc, w
    if par == 6:                                              # kep06.model:2-4
        P, A, phase, ecc, w = v
        return np.exp(P), A, phase, None, ecc, w
    raise ValueError(f'parameterisation {par} not supported')


class OracleRV:
    """The generated ``my_model`` / ``my_likelihood`` / ``my_prior`` of one run.

    ``spec`` is a model spec dict (module docstring), ``data`` the dict
    returned by :func:`preprocess`.
    """

    def __init__(self, spec, data):
        self.spec = spec
        self.blocks = spec['blocks']
        self.nins = int(spec['nins'])
        self.quirk = bool(spec.get('moav_reference_quirk', False))
        # run the reference's no-op per-instrument MA loop literally (timing)
        self.faithful_quirk_loop = bool(spec.get('faithful_quirk_loop', False))
        self.am = data.get('am') if any(b['type'] == 'AstrometryOffset' for b in self.blocks) else None
        # np.longdouble: the astrometric barycentre and scan-epoch propagation
        # in extended precision (oracle/am.py)
        self.am_dtype = np.float64
        self.X_ = np.asarray(data['X'], dtype=np.float64)
        self.Y_ = np.asarray(data['Y'], dtype=np.float64)
        self.YERR_ = np.asarray(data['YERR'], dtype=np.float64)
        flag = np.asarray(data['Flag'])
        self.ndat = len(self.X_)
        # emp_model.py:421-425
        self.masks = [flag == (n + 1) for n in range(self.nins)]
        self.ndats = [int(np.sum(m)) for m in self.masks]
        # 00.like:1
        self.likelihood_constant = - 0.5 * np.log(2 * np.pi) * self.ndat

        # global slices and fixed-parameter bookkeeping (emp_model.py:223-305)
        fixed, self.slices = [], []
        blen = 0
        for b in self.blocks:
            n = len(b['params'])
            self.slices.append(slice(blen, blen + n))
            blen += n
            fixed.extend(p.get('fixed') for p in b['params'])
        self.mod_fixed_ = np.array(fixed, dtype=object)
        free = np.array([f is None for f in fixed])
        self.C_ = np.arange(blen)[free]
        self.A_ = np.arange(blen)[~free]
        self.ndim = int(free.sum())
        # prior arguments after _check_prargs
        self.prior_terms = []          # per block: [(full index, fn, limits, args)]
        self.extra_terms = []          # per block: [(kind, fn, limits, args)]
        for b, sl in zip(self.blocks, self.slices):
            terms = []
            for i, p in enumerate(b['params']):
                if p.get('fixed') is not None:
                    continue
                args = check_prargs(p['prior'], p['limits'], p.get('prargs'))
                terms.append((sl.start + i, PRIORS[p['prior']], list(p['limits']), args))
            self.prior_terms.append(terms)
            extra = []
            for ap in b.get('additional', []):
                if not ap.get('has_prior'):
                    continue
                if ap['name'] == 'Hill':                 # emp.py:222-227
                    extra.append(('Hill', prior_Hill, list(ap['limits']), list(ap['prargs'])))
                    continue
                args = check_prargs(ap['prior'], ap['limits'], ap.get('prargs'))
                kind = ap['name'][:3]
                extra.append((kind, PRIORS[ap['prior']], list(ap['limits']), args))
            self.extra_terms.append(extra)

    # emp.py:190-192 / emp_model.py:709-711
    def full_theta(self, theta):
        theta = np.asarray(theta, dtype=np.float64)
        for a in self.A_:
            theta = np.insert(theta, a, self.mod_fixed_[a])
        return theta

    def my_model(self, theta):
        """Restates the generated ``my_model`` (emp_model.py:706-781)."""
        theta = self.full_theta(theta)
        X_, Y_ = self.X_, self.Y_
        model0 = np.zeros(self.ndat)
        err20 = self.YERR_ ** 2
        residuals = None
        for b, sl in zip(self.blocks, self.slices):
            t = b['type']
            if t == 'Keplerian':
                # an astrometric Keplerian's RV term is kep00's (akep00.model)
                per, A, phase, tp, ecc, w = kepler_elements(b['parameterisation'], theta[sl][:5])
                if tp is not None:                            # kep03/kep04: M = freq*(X_-tp)
                    freq = 2. * np.pi / per
                    M = freq * (X_ - tp)
                    E = kepler_solve(M, np.repeat(ecc, len(M)))
                    f = (np.arctan(((1. + ecc) ** 0.5 / (1. - ecc) ** 0.5) * np.tan(E / 2.)) * 2.)
                    model0 += A * (np.cos(f + w) + ecc * np.cos(w))
                else:
                    model0 += kepler_rv(X_, per, A, phase, ecc, w)
            elif t == 'Sinusoid':                              # sinusoid00.model:2-7
                per, A, phase = theta[sl]
                freq = 2. * np.pi / per
                M = freq * X_ + phase
                model0 += A * np.cos(M)
            elif t == 'MagneticCycle':                         # magneticcycle00.model:2-11
                per, A1, A2, phase1, phase2 = theta[sl]
                freq2 = 2. * np.pi / per
                freq1 = np.pi / per
                M1 = freq1 * X_ + phase1
                M2 = freq2 * X_ + phase2
                model0 += A1 * np.cos(M1) + A2 * np.cos(M2)
            elif t in ('Celerite2', 'AstrometryOffset', 'AstrometryJitter'):   # no RV model
                pass
            elif t == 'Acceleration':                          # acc.model:2
                model0 += np.polyval(np.concatenate([theta[sl], [0]]), (X_ - X_[0]))
            elif t == 'Offset':                                # offset00.model:3
                for nin in range(self.nins):
                    model0 += theta[sl][nin] * self.masks[nin]
            elif t == 'Jitter':                                # jitter00.model:3
                for nin in range(self.nins):
                    err20 += self.masks[nin] * theta[sl][nin] ** 2
            elif t == 'MOAV':                                  # emp_model.py:757-769
                residuals = Y_ - model0
                q = int(b['order'])
                if b['global']:
                    self._moav_global(theta[sl], q, model0, residuals)
                elif not self.quirk:
                    self._moav_per_instrument(theta[sl], q, model0, residuals)
                elif self.faithful_quirk_loop:
                    self._moav00_literal(theta[sl], q, model0, residuals)
                # quirk: moav00.model:18-19 writes through ``model0[mask][i]``,
                # a temporary copy, so the reference's per-instrument MA leaves
                # model0 unchanged.
            else:
                raise ValueError(f'block type {t} not in the hot path')
        return model0, err20

    def _moav_global(self, theta_ma, q, model0, residuals):
        """moav01.model:3-15 -- in-place recurrence over all epochs."""
        t_ = self.X_
        res_ = residuals
        for i in range(self.ndat):
            for c in range(q):
                if i > c:
                    dt = abs(t_[i] - t_[i - 1 - c])
                    macoef = theta_ma[2 * c]
                    matime = theta_ma[2 * c + 1]
                    MA = macoef * np.exp(-dt / matime) * res_[i - 1 - c]
                    model0[i] += MA
                    residuals[i] -= MA

    def _moav00_literal(self, theta_all, q, model0, residuals):
        """moav00.model:4-19 exactly as the reference runs it (timing only).

        Every ``model0[mask][i] += MA`` builds and discards a masked copy, so
        the loop costs O(ndat_k) per epoch and changes nothing.
        """
        for k in range(self.nins):
            mask = self.masks[k]
            t_ = self.X_[mask]
            res_ = residuals[mask]
            theta_ma = theta_all[q * 2 * k: q * 2 * (k + 1)]
            for c in range(q):
                macoef = theta_ma[2 * c]
                matime = theta_ma[2 * c + 1]
                for i in range(1, self.ndats[k]):
                    if i > c:
                        dt = abs(t_[i] - t_[i - 1 - c])
                        MA = macoef * np.exp(-dt / matime) * res_[i - 1 - c]
                        model0[mask][i] += MA
                        residuals[mask][i] -= MA

    def _moav_per_instrument(self, theta_all, q, model0, residuals):
        """The documented per-instrument MA(q) (docs/user-guide/ug-the-model.md:90-95).

        The recurrence of moav01.model:7-15 applied to each instrument's
        time-ordered subsequence, with that instrument's coefficients
        ``theta[slice][2q(k-1):2qk]`` (moav00.model:6).
        """
        for k in range(self.nins):
            idx = np.nonzero(self.masks[k])[0]
            theta_ma = theta_all[2 * q * k: 2 * q * (k + 1)]
            t_ = self.X_[idx]
            for ii in range(len(idx)):
                for c in range(q):
                    if ii > c:
                        dt = abs(t_[ii] - t_[ii - 1 - c])
                        MA = theta_ma[2 * c] * np.exp(-dt / theta_ma[2 * c + 1]) \
                            * residuals[idx[ii - 1 - c]]
                        model0[idx[ii]] += MA
                        residuals[idx[ii]] -= MA

    def my_likelihood(self, theta):
        """support/likelihoods/00.like:3-5; with a Celerite2 block
        support/likelihoods/02.like (oracle/gp.py)."""
        gp_terms = [b['gp_terms'] for b in self.blocks if b['type'] == 'Celerite2']
        if gp_terms:
            from . import gp
            model, err2 = self.my_model(theta)
            th = self.full_theta(theta)
            co = gp.coefficients([(k, [th[i] for i in sl]) for k, sl in gp_terms[0]])
            return gp.semisep_loglike(self.X_, self.Y_ - model, err2, co)
        model, err2 = self.my_model(theta)
        ll = -0.5 * (np.sum((self.Y_ - model) ** 2 / err2 + np.log(err2))) + self.likelihood_constant
        if self.am is not None:                          # support/likelihoods/a00.like
            from . import am as _am
            th = self.full_theta(theta)
            planets = [th[sl] for b, sl in zip(self.blocks, self.slices) if b['type'] == 'Keplerian']
            off = [th[sl] for b, sl in zip(self.blocks, self.slices) if b['type'] == 'AstrometryOffset'][0]
            jit = [th[sl] for b, sl in zip(self.blocks, self.slices) if b['type'] == 'AstrometryJitter'][0]
            ll = float(ll + _am.loglike_am(self.am, planets, off, jit, dtype=self.am_dtype))
        return ll

    def my_prior(self, theta):
        """Restates the generated ``my_prior`` (emp.py:182-254)."""
        theta = self.full_theta(theta)
        lp = 0.
        for b, sl, terms, extra in zip(self.blocks, self.slices,
                                       self.prior_terms, self.extra_terms):
            for j, fn, limits, args in terms:
                lp += fn(theta[j], limits, args)
            if lp == -np.inf:
                return lp
            for kind, fn, limits, args in extra:
                if kind == 'Amp':
                    x = theta[sl][1] ** 2 + theta[sl][2] ** 2
                elif kind == 'Ecc':
                    x = theta[sl][3] ** 2 + theta[sl][4] ** 2
                elif kind == 'Hill' and args[0] > 1:
                    x = hill_x(b['parameterisation'], theta, len(b['params']), int(args[0]))
                else:
                    continue
                lp += fn(x, limits, args)
        return lp

    def log_posterior(self, theta, beta=1.0):
        """(logL, logprior) with logL skipped when the prior is -inf."""
        lp = self.my_prior(theta)
        if not np.isfinite(lp):
            return -np.inf, lp
        return self.my_likelihood(theta), lp


# --------------------------------------------------------------------------
# reference-faithful script-level globals, for Pool mapping (the generated
# script defines my_likelihood / my_prior at module level; workers inherit
# them by fork, support/pools/01.pool:10-12)
# --------------------------------------------------------------------------
_GLOBAL = {}


def install_global(spec, data):
    _GLOBAL['oracle'] = OracleRV(spec, data)


def global_logpost(theta):
    o = _GLOBAL['oracle']
    lp = o.my_prior(theta)
    if lp == -np.inf:
        return -np.inf, lp
    return o.my_likelihood(theta), lp


def normal_logZ(low, high, mu, s):
    """ln(Phi(b) - Phi(a)) with math.erf (used by fixtures)."""
    a, b = (low - mu) / s, (high - mu) / s
    return math.log(0.5 * (math.erf(b / math.sqrt(2)) - math.erf(a / math.sqrt(2))))
