"""Post-run reductions on the device (emp_ladder_sums, emp_autocorr) against
the same estimators on host copies of the histories (stats.py): the
thermodynamic-integration and stepping-stone log-evidence and the
integrated autocorrelation time that EMPEROR's postprocess reads
(src/astroemperor/emp.py:1372-1447)."""
import numpy as np
import pytest

from astroemperor_gb300.engine import PTSampler
from astroemperor_gb300.stats import integrated_time, stepping_stone, thermodynamic_integration
from tests.golden.cases import model_51peg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def run(peg_arr, lib, cuda):
    m, d = model_51peg(peg_arr, k=1, par=1)
    T, W = 5, 32
    rng = np.random.default_rng(3)
    lim = m.limits_free()
    p0 = rng.uniform(lim[:, 0], lim[:, 1], size=(T, W, m.ndim__))
    p0[..., 0] = rng.uniform(4.225, 4.235, size=(T, W))
    p0[..., 3:5] *= 0.3
    s = PTSampler(W, m.ndim__, m, ntemps=T, seed=31, adapt_tau=100)
    s.run_mcmc(p0, nsweeps=600)
    return s


@pytest.mark.parametrize('discard', [0, 150])
def test_evidence_reductions_equal_host_estimators(run, discard):
    s = run
    ll = s.get_log_like(discard=discard)
    for pchip in (True, False):
        dev = s.get_evidence_ti(discard=discard, pchip=pchip)
        host = thermodynamic_integration(s.betas, ll, pchip=pchip)
        np.testing.assert_allclose(dev, host, rtol=1e-12)
    dev = s.get_evidence_ss(discard=discard)
    host = stepping_stone(s.betas, ll)
    np.testing.assert_allclose(dev[0], host[0], rtol=1e-12)
    np.testing.assert_allclose(dev[1], host[1], rtol=1e-8)


@pytest.mark.parametrize('discard,thin', [(0, 1), (200, 1), (100, 3)])
def test_autocorr_time_equals_host_estimator(run, discard, thin):
    s = run
    dev = s.get_autocorr_time(discard=discard, thin=thin, quiet=True)
    ch = s.get_chain(discard=discard, thin=thin)
    host = np.array([integrated_time(ch[t], quiet=True) * thin for t in range(s.ntemps)])
    np.testing.assert_allclose(dev, host, rtol=1e-5)
    assert dev.shape == (s.ntemps, s.ndim)
    with pytest.raises(RuntimeError):
        s.get_autocorr_time(discard=discard, thin=thin, tol=10 ** 6)
