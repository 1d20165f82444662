"""Pin the CPU oracle against numbers the reference recorded for 51 Peg.

The reference ships no unit tests and no single-theta vectors.  Its example
notebook ``tests/01_51peg_basic.ipynb`` records, for the 51 Peg data set:

* ``t0 epoch is : 2450002.665695`` (qol_utils.py:192-198 common_t);
* the default jitter limits ``[1e-05, 75.852]`` (max |RV - mean|,
  block_repo.py:710-722);
* k=0 (offset + jitter): best fit offset -0.148, jitter 36.064, maximum
  posterior -1333.617 and ``like_max`` -1308.794;
* k=1 (parameterisation 1, P in [3,5], K in [45,60], offset in [-10,10],
  jitter limits constrained to [1e-5, 40.600]): maximum posterior -881.725,
  ``like_max`` -869.493.

``like_max`` is the log-likelihood at the maximum-posterior sample
(``emp.py:1468-1469``), not the maximum of the likelihood.

The notebooks were recorded before the truncation normaliser ``logZ``
entered ``support/priors/Normal.prior`` (the line without it is still there,
commented out): their ``post_max - like_max`` equals the oracle's prior
plus the jitter prior's ``logZ``.  The posterior pins below therefore use
``prior + logZ``; the current prior is pinned by the normaliser formula of
``emp_model.py:90-94``.
"""
import numpy as np
import pytest
from scipy.optimize import minimize
from scipy.stats import norm

from oracle.rv import OracleRV, check_prargs, kepler_solve, preprocess, read_vels_folder
from tests.golden.cases import PEG_MAP_P1, model_51peg

JIT_K1 = [1e-5, 40.60023260950122]   # limits printed for the k=1 run


def test_preprocessing_pins(peg_arr):
    d = preprocess([peg_arr])
    assert d['common_t'] == pytest.approx(2450002.665695, abs=5e-7)
    assert len(d['X']) == 256
    assert d['X'][0] == 0.0
    assert np.max(np.abs(d['Y'])) == pytest.approx(75.852, abs=5e-4)
    assert abs(np.mean(d['Y'])) < 1e-12


def _oracle(peg_arr, k, jit=None):
    m, data = model_51peg(peg_arr, k=k, par=1)
    if jit is not None:
        m.blocks[-1][0].limits = list(jit)
    o = OracleRV(m.spec(), data.as_dict())
    lim = m.blocks[-1][0].limits
    logZ = check_prargs('Normal', lim, [5, 5])[2]
    return o, logZ


def _argmax(f, x0):
    r = minimize(lambda x: -f(x), x0, method='Nelder-Mead',
                 options=dict(xatol=1e-10, fatol=1e-11, maxiter=60000, maxfev=60000))
    r = minimize(lambda x: -f(x), r.x, method='Nelder-Mead',
                 options=dict(xatol=1e-10, fatol=1e-11, maxiter=60000, maxfev=60000))
    return -r.fun, r.x


def test_normal_prior_normaliser():
    lo, hi, mu, s = 1e-5, 75.852, 5.0, 5.0
    assert check_prargs('Normal', [lo, hi], [mu, s])[2] == pytest.approx(
        np.log(norm.cdf((hi - mu) / s) - norm.cdf((lo - mu) / s)), rel=1e-15)


def test_k0_pins(peg_arr):
    o, logZ = _oracle(peg_arr, 0)
    # like_max: logL at the recorded maximum-posterior fit
    assert o.my_likelihood([-0.148, 36.064]) == pytest.approx(-1308.794, abs=1e-3)
    post_nb = lambda x: o.my_likelihood(x) + o.my_prior(x) + logZ
    best, x = _argmax(post_nb, [-0.148, 36.064])
    assert best == pytest.approx(-1333.617, abs=2e-3)
    assert x[0] == pytest.approx(-0.148, abs=0.01) and x[1] == pytest.approx(36.064, abs=0.01)
    assert np.log(256) * 2 - 2 * o.my_likelihood(x) == pytest.approx(2628.678, abs=0.01)


def test_k1_pins(peg_arr):
    o, logZ = _oracle(peg_arr, 1, JIT_K1)
    # the prior at the recorded fit equals the recorded post_max - like_max
    assert o.my_prior(PEG_MAP_P1) + logZ == pytest.approx(-881.725 + 869.493, abs=2e-3)

    def post_nb(x):
        lp = o.my_prior(x)
        return o.my_likelihood(x) + lp + logZ if np.isfinite(lp) else -1e300
    best, x = _argmax(post_nb, PEG_MAP_P1)
    # the sampled maximum lies at or just below the true maximum
    assert -881.725 - 1e-3 <= best < -881.725 + 0.1, best
    assert o.my_likelihood(x) == pytest.approx(-869.493, abs=0.1)
    assert x[0] == pytest.approx(4.231, abs=1e-3)
    assert x[1] == pytest.approx(55.957, abs=0.3)
    assert x[5] == pytest.approx(3.642, abs=0.3)
    assert x[6] == pytest.approx(2.961, abs=0.3)


def test_kepler_solver_residual():
    rng = np.random.default_rng(0)
    M = rng.uniform(-50, 50, 20000)
    e = rng.uniform(0, 0.999, 20000)
    E = kepler_solve(M, e)
    Mr = np.remainder(M + np.pi, 2 * np.pi) - np.pi
    assert np.max(np.abs(E - e * np.sin(E) - Mr)) < 5e-15


def test_read_vels_folder(tmp_path, peg_arr):
    np.savetxt(tmp_path / 'a.vels', peg_arr)
    arrs, names = read_vels_folder(str(tmp_path))
    assert names == ['a.vels'] and np.allclose(arrs[0], peg_arr)
