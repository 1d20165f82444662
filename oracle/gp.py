"""Celerite Gaussian-process likelihood of the reference's GP runs
(oracle; TEST INFRASTRUCTURE ONLY).

The reference's GP path (``support/likelihoods/02.like``,
``support/kernels/00.kernel``, ``emp.py:341-412``) builds a celerite2 kernel
from ``cterms`` terms whose hyperparameters come from theta, sets
``gp.mean = model``, ``gp.compute(X_, diag=err2, quiet=True)`` and returns
``gp.log_likelihood(Y_)``.  celerite2 is a third-party dependency that the
reference does not pin and that is absent here; this module restates the
published definitions of the terms it uses (celerite2 0.3 ``terms``:
``RealTerm``, ``SHOTerm``, ``Matern32Term``, ``RotationTerm``, and the
reference's two-SHO ``GonzRotationTerm`` of ``emp.py:397-412``) as the
coefficients (a, b, c, d) of k(tau) = sum_j exp(-c_j tau) (a_j cos(d_j tau) +
b_j sin(d_j tau)), and evaluates the Gaussian log-likelihood two ways:
``dense_loglike`` (the definition: a dense covariance and its Cholesky
factor) and ``semisep_loglike`` (the O(N J^2) recursion of Foreman-Mackey,
Agol, Ambikasaran & Angus 2017, AJ 154, 220, which the device implements).
Parity with celerite2 itself is unpinned: neither the library nor outputs
of it are available.

``gp_semisep.c`` states the recursion in C (compiled here with gcc on first
use); ``use_compiled(True)`` routes ``semisep_loglike`` through it, which the
CPU baseline does so that a host evaluation costs what celerite2's compiled
core costs.  The tests check the two against each other.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, 'gp_semisep.c')
_LIB = os.path.join(_HERE, '_build', 'libgp_oracle.so')
_c = None
_use_c = False


def build_c():
    """Compile gp_semisep.c into oracle/_build (skipped when up to date)."""
    if os.path.exists(_LIB) and os.path.getmtime(_LIB) >= os.path.getmtime(_SRC):
        return _LIB
    os.makedirs(os.path.dirname(_LIB), exist_ok=True)
    tmp = _LIB + f'.{os.getpid()}.tmp'
    subprocess.run(['gcc', '-O2', '-shared', '-fPIC', '-o', tmp, _SRC, '-lm'], check=True)
    os.replace(tmp, _LIB)
    return _LIB


def _load_c():
    global _c
    if _c is None:
        lib = ctypes.CDLL(build_c())
        dp = ctypes.POINTER(ctypes.c_double)
        lib.emp_oracle_gp_loglike.restype = ctypes.c_double
        lib.emp_oracle_gp_loglike.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_int, dp, dp,
                                              ctypes.c_int, dp, dp, dp, dp]
        _c = lib
    return _c


def use_compiled(flag=True):
    """Route semisep_loglike through the compiled recursion (or back)."""
    global _use_c
    if flag:
        _load_c()
    _use_c = bool(flag)


def semisep_loglike_c(t, r, diag, coeffs):
    """semisep_loglike through gp_semisep.c."""
    lib = _load_c()
    ar, cr, a, b, c, d = (np.ascontiguousarray(x, dtype=np.float64) for x in coeffs)
    t, r, diag = (np.ascontiguousarray(x, dtype=np.float64) for x in (t, r, diag))
    dp = ctypes.POINTER(ctypes.c_double)
    P = lambda x: x.ctypes.data_as(dp)
    return float(lib.emp_oracle_gp_loglike(len(t), P(t), P(r), P(diag), len(ar), P(ar), P(cr),
                                           len(a), P(a), P(b), P(c), P(d)))

# term kinds of the compiled descriptor (include/emp_gpu.h, EMP_GP_*)
GP_REAL, GP_MATERN32, GP_ROTATION, GP_GROT = 1, 2, 3, 4
GP_SHO = 16          # + 1: amplitude given as sigma, + 2: frequency as rho, + 4: quality as tau

# parameter names of each term in canonical order, as keyword names of the
# celerite2 constructors (the reference's my_kernel['params'] keys)
TERM_KEYS = {
    'RealTerm': ('a', 'c'),
    'Matern32Term': ('sigma', 'rho'),
    'RotationTerm': ('sigma', 'period', 'Q0', 'dQ', 'f'),
    'GonzRotationTerm': ('rho', 'tau', 'A1', 'A2'),
}


def sho_kind(keys):
    """Descriptor kind and canonical key order of an SHOTerm keyword set."""
    keys = set(keys)
    amp = 'sigma' if 'sigma' in keys else 'S0'
    freq = 'rho' if 'rho' in keys else 'w0'
    qual = 'tau' if 'tau' in keys else 'Q'
    if {amp, freq, qual} != keys:
        raise ValueError(f'SHOTerm keywords {sorted(keys)} are not one of (S0|sigma, w0|rho, Q|tau)')
    kind = GP_SHO + (amp == 'sigma') + 2 * (freq == 'rho') + 4 * (qual == 'tau')
    return kind, (amp, freq, qual)


def sho_coefficients(S0=None, w0=None, Q=None, sigma=None, rho=None, tau=None, eps=1e-5):
    """celerite2 SHOTerm: (a_real, c_real, a, b, c, d)."""
    if w0 is None:
        w0 = 2 * np.pi / rho
    if Q is None:
        Q = 0.5 * w0 * tau
    if S0 is None:
        S0 = sigma ** 2 / (w0 * Q)
    if Q < 0.5:
        f = np.sqrt(max(1.0 - 4.0 * Q ** 2, eps))
        a = 0.5 * S0 * w0 * Q
        return ([a * (1 + 1 / f), a * (1 - 1 / f)], [0.5 * w0 / Q * (1 - f), 0.5 * w0 / Q * (1 + f)],
                [], [], [], [])
    f = np.sqrt(max(4.0 * Q ** 2 - 1.0, eps))
    a = S0 * w0 * Q
    return [], [], [a], [a / f], [0.5 * w0 / Q], [0.5 * w0 * f / Q]


def term_coefficients(kind, p):
    """(a_real, c_real, a, b, c, d) of one descriptor term with canonical
    parameters ``p``."""
    if kind == GP_REAL:
        return [p[0]], [p[1]], [], [], [], []
    if kind == GP_MATERN32:                        # celerite2 Matern32Term, eps = 0.01
        sigma, rho, eps = p[0], p[1], 0.01
        w0 = np.sqrt(3.0) / rho
        return [], [], [sigma ** 2], [sigma ** 2 * w0 / eps], [w0], [eps]
    if kind == GP_ROTATION:                        # celerite2 RotationTerm
        sigma, period, Q0, dQ, f = p[:5]
        amp = sigma ** 2 / (1 + f)
        Q1 = 0.5 + Q0 + dQ
        w1 = 4 * np.pi * Q1 / (period * np.sqrt(4 * Q1 ** 2 - 1))
        Q2 = 0.5 + Q0
        w2 = 8 * np.pi * Q2 / (period * np.sqrt(4 * Q2 ** 2 - 1))
        return _sum(sho_coefficients(S0=amp / (w1 * Q1), w0=w1, Q=Q1),
                    sho_coefficients(S0=f * amp / (w2 * Q2), w0=w2, Q=Q2))
    if kind == GP_GROT:                            # emp.py:404-405
        rho, tau, A1, A2 = p[:4]
        return _sum(sho_coefficients(S0=A1, rho=rho, tau=tau),
                    sho_coefficients(S0=A2, rho=rho * 0.5, tau=tau))
    if GP_SHO <= kind < GP_SHO + 8:
        bits = kind - GP_SHO
        kw = {('sigma' if bits & 1 else 'S0'): p[0], ('rho' if bits & 2 else 'w0'): p[1],
              ('tau' if bits & 4 else 'Q'): p[2]}
        return sho_coefficients(**kw)
    raise ValueError(f'GP term kind {kind} unknown')


def _sum(*cs):
    return tuple(sum((list(c[i]) for c in cs), []) for i in range(6))


def coefficients(terms):
    """Concatenated coefficients of [(kind, params), ...]."""
    return _sum(*[term_coefficients(k, p) for k, p in terms])


def kernel_value(coeffs, tau):
    ar, cr, a, b, c, d = (np.asarray(x, dtype=np.float64) for x in coeffs)
    tau = np.abs(np.asarray(tau, dtype=np.float64))[..., None]
    k = np.sum(ar * np.exp(-cr * tau), axis=-1) if len(ar) else 0.0
    if len(a):
        k = k + np.sum(np.exp(-c * tau) * (a * np.cos(d * tau) + b * np.sin(d * tau)), axis=-1)
    return k


def dense_loglike(t, r, diag, coeffs):
    """-0.5 (r^T K^-1 r + log det K + N log 2 pi), K = k(|t_i - t_j|) + diag;
    -inf when K is not positive definite."""
    t = np.asarray(t, dtype=np.float64)
    K = kernel_value(coeffs, t[:, None] - t[None, :])
    K[np.diag_indices_from(K)] += diag
    try:
        L = np.linalg.cholesky(K)
    except np.linalg.LinAlgError:
        return -np.inf
    z = np.linalg.solve(L, r)
    return float(-0.5 * (z @ z) - np.sum(np.log(np.diag(L))) - 0.5 * len(t) * np.log(2 * np.pi))


def semisep_loglike(t, r, diag, coeffs):
    """The same log-likelihood by the celerite recursion: with
    U_n = [a cos(d t_n) + b sin(d t_n), a sin(d t_n) - b cos(d t_n)],
    V_n = [cos(d t_n), sin(d t_n)] per term (real terms: d = b = 0) and
    phi_n = exp(-c (t_n - t_{n-1})):
      S_n = phi_n (S_{n-1} + D_{n-1} W_{n-1} W_{n-1}^T) phi_n,
      D_n = A_n - U_n^T S_n U_n,  W_n = (V_n - S_n U_n) / D_n,
      f_n = phi_n (f_{n-1} + W_{n-1} z_{n-1}),  z_n = r_n - U_n^T f_n,
    logL = -0.5 sum(z_n^2 / D_n + log D_n) - 0.5 N log 2 pi."""
    if _use_c:
        return semisep_loglike_c(t, r, diag, coeffs)
    ar, cr, a, b, c, d = (np.asarray(x, dtype=np.float64) for x in coeffs)
    A = np.concatenate([ar, a])
    Bc = np.concatenate([np.zeros_like(ar), b])
    C = np.concatenate([cr, c])
    Dd = np.concatenate([np.zeros_like(ar), d])
    J = len(A)
    t = np.asarray(t, dtype=np.float64)
    diag0 = np.sum(A)
    S = np.zeros((2 * J, 2 * J))
    f = np.zeros(2 * J)
    W = np.zeros(2 * J)
    Dprev, zprev = 0.0, 0.0
    quad, logdet = 0.0, 0.0
    for n in range(len(t)):
        cd, sd = np.cos(Dd * t[n]), np.sin(Dd * t[n])
        U = np.concatenate([A * cd + Bc * sd, A * sd - Bc * cd])
        V = np.concatenate([cd, sd])
        if n > 0:
            ph = np.tile(np.exp(-C * (t[n] - t[n - 1])), 2)
            S = ph[:, None] * (S + Dprev * np.outer(W, W)) * ph[None, :]
            f = ph * (f + W * zprev)
        Dn = diag[n] + diag0 - U @ S @ U
        if not Dn > 0:
            return -np.inf
        W = (V - S @ U) / Dn
        zn = r[n] - U @ f
        quad += zn * zn / Dn
        logdet += np.log(Dn)
        Dprev, zprev = Dn, zn
    return float(-0.5 * (quad + logdet) - 0.5 * len(t) * np.log(2 * np.pi))
