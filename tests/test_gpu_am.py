"""Joint RV + astrometry likelihood (support/likelihoods/a00.like) on the
GPU against the oracle, which tests/test_am_oracle.py pins to the
reference's own generated astrometry functions: the HIP 21850 model of the
reference's tests/03_hip21850_test.ipynb.

The reference's formulas handle absolute positions in degrees, whose FP64
rounding (2.5e-8 mas per ulp of 60 degrees) moves the Gaia term by up to
~4e-9 of the total log-likelihood (measured: the FP64 oracle, which equals
the reference's own functions to 1e-12, against the same formulas with the
propagation in long double).  The device forms the scan positions as offsets
from the DR3 position and is compared with the long-double value:
FP64 logL relative 5e-10 (the astrometric term is FP64; the mixed precision
solves its Kepler equations in FP32 with a float-float correction, E to ~1e-11;
what remains is the Hipparcos-epoch barycentre, propagated through absolute
angles as the reference does, where one ulp moves the Hipparcos term by up
to 5.4e-11 of the total; measured 1.1e-10), mixed 1e-6, logprior 1e-13 (the
Isotropic inclination prior included).  The PT sampler with the astrometric
term walks the oracle sampler's chain (same Philox stream; the oracle's
astrometric term in long double).
"""
import os

import numpy as np
import pytest
import torch

from astroemperor_gb300 import _native as N
from astroemperor_gb300.engine import Context, PTSampler
from oracle.pt import OraclePT
from oracle.rv import OracleRV
from tests.golden.cases import HIP_MAP, model_hip21850

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


@pytest.fixture(scope='module')
def hip(lib, cuda):
    fix = np.load(os.path.join(GOLDEN, 'hip21850.npz'))
    model, data, am = model_hip21850(fix)
    return model, data, am, Context(model, 'cuda:0')


def _case(planets):
    """(model, context, fixture arrays) of the one- or two-planet case"""
    fix = np.load(os.path.join(GOLDEN, 'hip21850.npz'))
    model, data, am = model_hip21850(fix, planets)
    pre = '' if planets == 1 else 'k2__'
    k = {key[len(pre):]: v for key, v in np.load(os.path.join(GOLDEN, 'am_kat.npz')).items()
         if key.startswith(pre) and (pre or not key.startswith('k2__'))}
    return model, Context(model, 'cuda:0'), k


@pytest.mark.parametrize('planets', [1, 2])
@pytest.mark.parametrize('prec,tol', [(N.EMP_PREC_FP64, 5e-10), (N.EMP_PREC_MIXED, 1e-6)])
def test_logpost_matches_the_oracle(lib, cuda, planets, prec, tol):
    model, ctx, k = _case(planets)
    th = k['theta']
    ll, lp = ctx.logpost(torch.as_tensor(th, device='cuda:0'), precision=prec)
    torch.cuda.synchronize()
    ll, lp = ll.cpu().numpy(), lp.cpu().numpy()
    np.testing.assert_allclose(lp, k['logprior'], rtol=1e-13, atol=1e-13)
    fin = np.isfinite(k['logprior'])
    assert np.all(ll[~fin] == -np.inf)
    ld = k['logl_ld'][fin]
    rel = np.abs(ll[fin] - ld) / np.abs(ld)
    ref_noise = np.abs(k['logl'][fin] - ld) / np.abs(ld)
    print(f'astrometry + RV logL against the long-double value: max relative error {rel.max():.2e} '
          f'(the FP64 reference formulas: {ref_noise.max():.2e})')
    assert rel.max() <= tol


def test_pt_replay_matches_the_oracle_sampler(hip):
    model, data, am, ctx = hip
    T, W, S = 3, 16, 8
    betas = [1.0, 0.3, 0.05]
    rng = np.random.default_rng(7)
    lim = model.limits_free()
    p0 = np.clip(np.array(HIP_MAP) + 1e-3 * (lim[:, 1] - lim[:, 0]) * rng.normal(size=(T, W, len(HIP_MAP))),
                 lim[:, 0], lim[:, 1])
    s = PTSampler(W, model.ndim__, model, ntemps=T, betas=betas, precision='fp64', seed=2024,
                  adapt_tau=20, use_graph=False, context=ctx, autotune=False)
    s.run_mcmc(p0, nsweeps=S)
    o = OracleRV(model.spec(), dict(data.as_dict(), am=am.as_dict()))
    o.am_dtype = np.longdouble

    def f(th):
        th = np.atleast_2d(th)
        lp = np.array([o.my_prior(t) for t in th])
        ll = np.array([o.my_likelihood(t) if np.isfinite(x) else -np.inf for t, x in zip(th, lp)])
        return ll, lp
    ora = OraclePT(f, T, W, model.ndim__, betas, adapt=True, adapt_tau=20, rng='philox', seed=2024)
    ora.set_positions(p0)
    ora.run(S)
    np.testing.assert_allclose(s.get_chain(), np.moveaxis(np.array(ora.chain), 1, 0), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(s.get_log_like(), np.moveaxis(np.array(ora.log_like), 1, 0), rtol=5e-10)
    assert ora.accepted.sum() > 0


def test_graph_equals_eager(hip):
    model, data, am, ctx = hip
    T, W = 2, 16
    rng = np.random.default_rng(9)
    lim = model.limits_free()
    p0 = np.clip(np.array(HIP_MAP) + 1e-3 * (lim[:, 1] - lim[:, 0]) * rng.normal(size=(T, W, len(HIP_MAP))),
                 lim[:, 0], lim[:, 1])
    out = []
    for ug in (False, True):
        s = PTSampler(W, model.ndim__, model, ntemps=T, betas=[1.0, 0.2], precision='mixed', seed=5,
                      use_graph=ug, context=ctx, autotune=False)
        s.run_mcmc(p0, nsweeps=20)
        out.append((s.get_chain(), s.get_log_like()))
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)


def test_gradient_refuses_astrometry(hip):
    model, data, am, ctx = hip
    th = torch.as_tensor(np.array([HIP_MAP]), device='cuda:0')
    with pytest.raises(N.EmpError) as e:
        ctx.logpost_grad(th)
    assert e.value.code == N.EMP_E_UNSUPPORTED
