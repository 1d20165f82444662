"""The FP64 torch autograd reference of the log-likelihood (the checker of
the adjoint kernel) against the oracle, on the CPU: equal log-likelihoods on
the golden cases of every parameterisation, trend block and MA form, and
gradients equal to central differences of the oracle (Richardson-extrapolated,
so that the period components, whose second derivatives are large, are
checked too)."""
import numpy as np
import pytest
import torch

from oracle.grad_ref import TorchRV
from oracle.rv import OracleRV
from tests.golden.cases import kat_case_models

CASES = ['51peg_k0', '51peg_k1_p0', '51peg_k1_p1', '51peg_k1_p2', '51peg_k1_p3', '51peg_k1_p4',
         '51peg_k1_p6', '51peg_k1_p7', '51peg_fixed_acc', '51peg_gma2', '51peg_k1_sin',
         '51peg_k1_cycle_gma1', '51peg_k2_hill', '51peg_ma2_inst', 'c2_ma1', 'c2_ma1_quirk']


def _finite(o, th):
    with np.errstate(all='ignore'):
        return np.array([t for t in th if np.isfinite(o.my_prior(t))])


@pytest.mark.parametrize('name', CASES)
def test_torch_reference_equals_oracle(peg_arr, name):
    m, d, th = kat_case_models(peg_arr)[name]
    o = OracleRV(m.spec(), d.as_dict())
    good = _finite(o, th)[:8]
    ll, g = TorchRV(m.spec(), d.as_dict()).grad(good)
    want = np.array([o.my_likelihood(t) for t in good])
    np.testing.assert_allclose(ll, want, rtol=1e-12)
    assert np.all(np.isfinite(g))


@pytest.mark.parametrize('name', ['51peg_k1_p0', '51peg_k1_p1', '51peg_k1_p2', '51peg_k1_p3', '51peg_k1_p4',
                                  '51peg_k1_p6', '51peg_k1_p7', '51peg_k1_sin', '51peg_k1_cycle_gma1',
                                  '51peg_fixed_acc', 'c2_ma1'])
def test_torch_gradient_equals_central_differences(peg_arr, name):
    m, d, th = kat_case_models(peg_arr)[name]
    o = OracleRV(m.spec(), d.as_dict())
    good = _finite(o, th)
    # points near the fit, where the chain is most curved
    x = good[-3] if len(good) > 3 else good[0]
    _, g = TorchRV(m.spec(), d.as_dict()).grad(x[None, :])
    lim = m.limits_free()
    for j in range(len(x)):
        def D(hh):
            a, c = x.copy(), x.copy()
            a[j] += hh
            c[j] -= hh
            return (o.my_likelihood(a) - o.my_likelihood(c)) / (2 * hh)
        # Richardson estimates at decreasing steps; the pair that agrees best
        # (truncation gone, rounding not yet dominant) gives the derivative
        hs = [10.0 ** -k * (lim[j, 1] - lim[j, 0]) for k in range(5, 10)]
        R = [(4 * D(h / 2) - D(h)) / 3 for h in hs]
        k = int(np.argmin([abs(R[i] - R[i + 1]) for i in range(len(R) - 1)]))
        fd = 0.5 * (R[k] + R[k + 1])
        assert g[0, j] == pytest.approx(fd, rel=1e-5, abs=1e-6 * np.max(np.abs(g)) + abs(R[k] - R[k + 1])), \
            (name, j)
