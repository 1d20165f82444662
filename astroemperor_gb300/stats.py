"""Post-run estimators the reference asks of its sampler.

* ``integrated_time`` -- emcee's integrated autocorrelation time estimator
  (Sokal's automated windowing with constant ``c``), which EMPEROR reads
  through ``sampler.get_autocorr_time`` (``src/astroemperor/emp.py:1372-1385``).
* ``thermodynamic_integration`` -- log-evidence by integrating the mean
  log-likelihood over the inverse-temperature ladder, which EMPEROR reads
  through ``sampler.get_evidence_ti`` (``emp.py:1432-1447``).
* ``stepping_stone`` -- log-evidence by the stepping-stone estimator of
  Xie, Lewis, Fan, Kuo & Chen (2011, Syst. Biol. 60, 150), read through
  ``sampler.get_evidence_ss`` when EMPEROR's ``evidence_method`` is 'ss'
  (``emp.py:1431-1441``).
* ``model_stats`` -- chi2, AIC, BIC, HQIC, RMSE of a fit (``emp.py:1187-1210``).
* ``hdi_of_samples`` / ``hdi_of_chain`` -- highest-density intervals of the
  posterior summaries (``math_utils.py:72-105``).

The sampler reduces its histories on the device (``emp_ladder_sums``,
``emp_autocorr``); ``ti_from_means``, ``ss_from_sums`` and ``tau_from_acf``
finish the estimators from those summaries, and the array forms above are
the same estimators on host arrays.
"""
from __future__ import annotations

import numpy as np


def _next_pow_two(n):
    i = 1
    while i < n:
        i <<= 1
    return i


def autocorr_1d(x):
    x = np.atleast_1d(x).astype(np.float64)
    n = _next_pow_two(len(x))
    f = np.fft.fft(x - np.mean(x), n=2 * n)
    acf = np.fft.ifft(f * np.conjugate(f))[: len(x)].real
    if acf[0] == 0:
        return np.ones_like(acf)
    return acf / acf[0]


def _auto_window(taus, c):
    m = np.arange(len(taus)) < c * taus
    if np.any(m):
        return int(np.argmin(m))
    return len(taus) - 1


def tau_from_acf(f, c=5):
    """(tau, window found) from a walker-averaged autocorrelation f [lags]:
    taus = 2 cumsum(f) - 1, the window the first lag m with m >= c taus[m]
    (Sokal's automated windowing).  ``found`` is False when no lag of f
    satisfies it (then tau is taken at the last lag, as emcee does for the
    full series)."""
    taus = 2.0 * np.cumsum(f) - 1.0
    m = np.arange(len(taus)) < c * taus
    if np.any(~m):
        return float(taus[int(np.argmin(m))]), True
    return float(taus[-1]), False


def check_tau(tau, n_t, tol=50, quiet=False):
    if tol > 0 and np.any(tol * np.asarray(tau) > n_t):
        msg = (f'the chain is shorter than {tol} times the integrated autocorrelation '
               f'time; N/{tol} = {n_t / tol:.0f}, tau = {tau}')
        if not quiet:
            raise RuntimeError(msg)


def integrated_time(x, c=5, tol=50, quiet=False):
    """tau per parameter of a chain x [steps, walkers, ndim] (host; the
    sampler computes the autocorrelation on the device, emp_autocorr)."""
    x = np.asarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x[:, None, None]
    if x.ndim == 2:
        x = x[:, :, None]
    n_t, n_w, n_d = x.shape
    tau = np.empty(n_d)
    for d in range(n_d):
        f = np.zeros(n_t)
        for k in range(n_w):
            f += autocorr_1d(x[:, k, d])
        f /= n_w
        tau[d] = tau_from_acf(f, c)[0]
    check_tau(tau, n_t, tol, quiet)
    return tau


def thermodynamic_integration(betas, log_like, pchip=True):
    """(logZ, error) from <log L> per temperature.

    ``log_like`` is [ntemps, steps, walkers] (or [ntemps, n]).  The ladder
    is completed with beta = 0 (taking the hottest chain's mean) when it
    does not reach it; the error is the difference between the full-ladder
    and the every-other-rung estimates.
    """
    betas = np.asarray(betas, dtype=np.float64)
    ll = np.asarray(log_like, dtype=np.float64).reshape(len(betas), -1)
    mean = np.array([np.mean(r[np.isfinite(r)]) if np.any(np.isfinite(r)) else -np.inf for r in ll])
    return ti_from_means(betas, mean, pchip)


def ti_from_means(betas, mean, pchip=True):
    """``thermodynamic_integration`` from the per-temperature means."""
    betas = np.asarray(betas, dtype=np.float64)
    mean = np.asarray(mean, dtype=np.float64)
    order = np.argsort(betas)
    b, m = betas[order], mean[order]
    if b[0] > 0:
        b = np.concatenate([[0.0], b])
        m = np.concatenate([[m[0]], m])

    def integ(bb, mm):
        if pchip and len(bb) > 2:
            try:
                from scipy.interpolate import PchipInterpolator
                return float(PchipInterpolator(bb, mm).integrate(bb[0], bb[-1]))
            except Exception:
                pass
        return float(np.trapezoid(mm, bb))

    z = integ(b, m)
    if len(b) > 3:
        z2 = integ(b[::2] if b[-1] == b[::2][-1] else np.append(b[::2], b[-1]),
                   m[::2] if b[-1] == b[::2][-1] else np.append(m[::2], m[-1]))
        err = abs(z - z2)
    else:
        err = np.inf
    return z, err


def stepping_stone(betas, log_like):
    """(logZ, error) by stepping stones between adjacent inverse temperatures.

    With the ladder sorted 0 <= b_0 < ... < b_K = 1 and samples L_i of the
    log-likelihood drawn at b_{k-1}, each stone is
    r_k = mean_i exp((b_k - b_{k-1}) L_i), and log Z = sum_k log r_k (each
    mean taken with a log-sum-exp shift).  A ladder that stops above zero is
    closed by thermodynamic integration of the hottest chain's mean over
    [0, b_0].  The error is the delta-method standard deviation of the
    summed log r_k, treating the samples of each rung as independent.
    """
    betas = np.asarray(betas, dtype=np.float64)
    ll = np.asarray(log_like, dtype=np.float64).reshape(len(betas), -1)
    order = np.argsort(betas)
    b, rows = betas[order], ll[order]
    logz, var = 0.0, 0.0
    hot = rows[0][np.isfinite(rows[0])]
    if b[0] > 0:
        if hot.size == 0:
            return -np.inf, np.inf
        logz += b[0] * float(np.mean(hot))
    for k in range(1, len(b)):
        x = rows[k - 1]
        x = x[np.isfinite(x)]
        if x.size == 0:
            return -np.inf, np.inf
        a = (b[k] - b[k - 1]) * x
        m = float(np.max(a))
        w = np.exp(a - m)
        mw = float(np.mean(w))
        logz += m + np.log(mw)
        if x.size > 1:
            var += float(np.var(w, ddof=1)) / (x.size * mw * mw)
    return float(logz), float(np.sqrt(var))


def hdi_of_samples(samples, cred_mass=0.9):
    """Shortest interval holding ``cred_mass`` of the samples
    (``src/astroemperor/math_utils.py:72-85``): over the sorted samples, the
    window of floor(cred_mass * n) steps with the least width."""
    s = np.sort(np.asarray(samples, dtype=np.float64))
    n = len(s)
    k = int(np.floor(cred_mass * n))
    widths = s[k:] - s[: n - k]
    i = int(np.argmin(widths))
    return s[i], s[i + k]


def hdi_of_chain(chain, cred_mass=0.9):
    """``hdi_of_samples`` per column of a flat chain [n, ndim] -> [ndim, 2]
    (``math_utils.py:88-105``)."""
    chain = np.asarray(chain, dtype=np.float64)
    return np.array([hdi_of_samples(chain[:, j], cred_mass) for j in range(chain.shape[1])])


def model_stats(residuals, err2, ndim, like_max, flags=None, nins=1):
    n = len(residuals)
    out = {}
    out['chi2'] = float(np.sum(residuals ** 2 / err2))
    out['chi2_red'] = out['chi2'] / (n - ndim)
    out['RMSE'] = float(np.sqrt(np.sum(residuals ** 2) / n))
    out['dof'] = n - ndim
    if flags is not None:
        out['RMSi'] = [float(np.sqrt(np.mean(residuals[flags == i + 1] ** 2))) for i in range(nins)]
        # emp.py:1195-1197 weighs each instrument by len(FLAGS_ == k) / RMSi**2,
        # where the length is that of the whole boolean mask (n for every k)
        w = np.array([n / r ** 2 for r in out['RMSi']])
        out['Weights'] = w / np.sum(w)
    out['AIC'] = 2 * ndim - 2 * like_max
    out['BIC'] = np.log(n) * ndim - 2 * like_max
    out['HQIC'] = 2 * ndim * np.log(np.log(n)) - 2 * like_max
    return out


def stepping_stone_plan(betas):
    """The stones of ``stepping_stone``: (order of the ladder ascending in
    beta, source temperature of each stone, its beta step)."""
    betas = np.asarray(betas, dtype=np.float64)
    order = np.argsort(betas)
    b = betas[order]
    src = np.array([order[k - 1] for k in range(1, len(b))], dtype=np.int32)
    step = np.array([b[k] - b[k - 1] for k in range(1, len(b))], dtype=np.float64)
    return order, src, step


def ss_from_sums(betas, temp_sums, stone_sums):
    """``stepping_stone`` from the device summaries: temp_sums [T][2] (sum,
    count of finite log L per temperature) and stone_sums [K][4] (max of
    d L, sum exp(d L - max), sum of its square, count) of the stones of
    ``stepping_stone_plan``."""
    betas = np.asarray(betas, dtype=np.float64)
    order, src, step = stepping_stone_plan(betas)
    b0 = betas[order[0]]
    logz, var = 0.0, 0.0
    if b0 > 0:
        s, n = temp_sums[order[0]]
        if n == 0:
            return -np.inf, np.inf
        logz += b0 * s / n
    for m, s1, s2, n in stone_sums:
        if n == 0:
            return -np.inf, np.inf
        mw = s1 / n
        logz += m + np.log(mw)
        if n > 1:
            vw = (s2 - n * mw * mw) / (n - 1)
            var += max(vw, 0.0) / (n * mw * mw)
    return float(logz), float(np.sqrt(var))
