"""Post-run reductions on cases with known answers: evidence by
thermodynamic integration and by stepping stones on a Gaussian model with an
analytic evidence, and the integrated autocorrelation time of an AR(1)
series."""
import numpy as np
import pytest

from astroemperor_gb300.stats import integrated_time, stepping_stone, thermodynamic_integration


def _gaussian_ladder(n=4000, ntemps=24, seed=0):
    """Exact samples of logL at each inverse temperature of a 1-D model:
    prior N(0, s0^2), likelihood N(y | theta, s^2); Z = N(y | 0, s0^2 + s^2)."""
    rng = np.random.default_rng(seed)
    s0, s, y = 3.0, 0.5, 1.3
    betas = np.concatenate([[1.0], np.geomspace(0.5, 1e-6, ntemps - 1)])
    ll = []
    for b in betas:
        prec = 1 / s0 ** 2 + b / s ** 2
        mu = (b * y / s ** 2) / prec
        th = mu + rng.normal(size=n) / np.sqrt(prec)
        ll.append(-0.5 * (y - th) ** 2 / s ** 2 - 0.5 * np.log(2 * np.pi * s ** 2))
    v = s0 ** 2 + s ** 2
    logz = -0.5 * y ** 2 / v - 0.5 * np.log(2 * np.pi * v)
    return betas, np.array(ll), logz


def test_stepping_stone_recovers_analytic_evidence():
    betas, ll, logz = _gaussian_ladder()
    z, err = stepping_stone(betas, ll)
    assert err < 0.05
    assert z == pytest.approx(logz, abs=max(4 * err, 0.02))


def test_thermodynamic_integration_recovers_analytic_evidence():
    betas, ll, logz = _gaussian_ladder()
    z, err = thermodynamic_integration(betas, ll)
    assert z == pytest.approx(logz, abs=0.05)


def test_stepping_stone_handles_empty_rungs():
    betas = np.array([1.0, 0.1])
    ll = np.array([[-1.0, -2.0], [-np.inf, -np.inf]])
    assert stepping_stone(betas, ll)[0] == -np.inf


def test_integrated_time_of_ar1():
    rng = np.random.default_rng(3)
    phi, n, w = 0.8, 20000, 8
    x = np.zeros((n, w))
    e = rng.normal(size=(n, w))
    for i in range(1, n):
        x[i] = phi * x[i - 1] + e[i]
    tau = integrated_time(x[:, :, None])[0]
    assert tau == pytest.approx((1 + phi) / (1 - phi), rel=0.1)
