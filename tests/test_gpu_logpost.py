"""CUDA log-posterior against the oracle (through the C ABI).

Tolerances
  FP64 plain : logprior rel 1e-13; logL rel 1e-11 (summation order and
               libm ulps differ from numpy)
  mixed      : |dlogL| / |logL| <= 1e-6 at every theta with a finite prior
"""
import numpy as np
import pytest
import torch

from astroemperor_gb300 import _native as N
from astroemperor_gb300.engine import Context
from oracle.rv import OracleRV
from tests.golden.cases import kat_case_models

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-11
MIXED_RTOL = 1e-6


@pytest.fixture(scope='module')
def models(peg_arr, lib, cuda):
    return kat_case_models(peg_arr)


@pytest.fixture(scope='module')
def contexts(models, cuda):
    return {k: Context(m, 'cuda:0') for k, (m, d, th) in models.items()}


def _eval(ctx, th, prec):
    t = torch.as_tensor(th, dtype=torch.float64, device='cuda:0')
    ll, lp = ctx.logpost(t, precision=prec)
    torch.cuda.synchronize()
    return ll.cpu().numpy(), lp.cpu().numpy()


def test_fp64_matches_golden(models, contexts, kat):
    for name, (m, d, th) in models.items():
        ll, lp = _eval(contexts[name], th, N.EMP_PREC_FP64)
        klp, kll = kat[f'{name}__logprior'], kat[f'{name}__logl']
        np.testing.assert_allclose(lp, klp, rtol=1e-13, atol=1e-13, err_msg=name)
        fin = np.isfinite(klp)
        assert np.all(ll[~fin] == -np.inf), name
        np.testing.assert_allclose(ll[fin], kll[fin], rtol=FP64_RTOL, err_msg=name)


def test_mixed_within_tolerance(models, contexts, kat):
    worst = {}
    for name, (m, d, th) in models.items():
        ll, lp = _eval(contexts[name], th, N.EMP_PREC_MIXED)
        klp, kll = kat[f'{name}__logprior'], kat[f'{name}__logl']
        np.testing.assert_allclose(lp, klp, rtol=1e-13, atol=1e-13, err_msg=name)
        fin = np.isfinite(klp) & np.isfinite(kll)
        rel = np.abs(ll[fin] - kll[fin]) / np.abs(kll[fin])
        worst[name] = float(rel.max())
    print('mixed worst relative error per case:', worst)
    assert max(worst.values()) <= MIXED_RTOL, worst


@pytest.mark.parametrize('prec', [N.EMP_PREC_FP64, N.EMP_PREC_MIXED])
def test_launch_shapes_agree(models, contexts, prec):
    for name in ('c2_ma1', '51peg_gma2', '51peg_k1_p1'):
        m, d, th = models[name]
        ctx = contexts[name]
        ref, _ = _eval(ctx, th, prec)
        fin = np.isfinite(ref)
        for L in (8, 16, 32, 64, 128, 256):
            for tile in (0, 64, 200):
                ctx.set_launch(prec, L, tile)
                ll, _ = _eval(ctx, th, prec)
                tol = 1e-12 if prec == N.EMP_PREC_FP64 else 2e-7
                np.testing.assert_allclose(ll[fin], ref[fin], rtol=tol, err_msg=f'{name} L={L} tile={tile}')
                assert np.all(ll[~fin] == -np.inf)
        ctx.set_launch(prec, 0, 0)


def test_batch_sizes_and_empty(models, contexts):
    m, d, th = models['51peg_k1_p1']
    ctx = contexts['51peg_k1_p1']
    ref, _ = _eval(ctx, th, N.EMP_PREC_FP64)
    for B in (1, 3, 17):
        ll, _ = _eval(ctx, th[:B], N.EMP_PREC_FP64)
        np.testing.assert_array_equal(ll, ref[:B])
    t0 = torch.zeros(0, m.ndim__, dtype=torch.float64, device='cuda:0')
    ll, lp = ctx.logpost(t0, precision=N.EMP_PREC_FP64)
    assert ll.numel() == 0


def test_nan_theta_gives_minus_inf(models, contexts):
    m, d, th = models['51peg_k1_p1']
    bad = th[:4].copy()
    bad[0, 0] = np.nan
    bad[1, 6] = np.inf
    ll, lp = _eval(contexts['51peg_k1_p1'], bad, N.EMP_PREC_MIXED)
    assert lp[0] == -np.inf and lp[1] == -np.inf and ll[0] == -np.inf and ll[1] == -np.inf


def test_model_eval_matches_oracle(models, contexts):
    for name in ('51peg_k1_p1', 'c2_ma1', 'c2_ma1_quirk', '51peg_gma2', '51peg_fixed_acc', '51peg_k1_p3',
                 '51peg_k1_sin', '51peg_k1_cycle_gma1'):
        m, d, th = models[name]
        o = OracleRV(m.spec(), d.as_dict())
        good = np.array([t for t in th if np.isfinite(o.my_prior(t))][:5])
        t = torch.as_tensor(good, dtype=torch.float64, device='cuda:0')
        model, err2 = contexts[name].model_eval(t)
        torch.cuda.synchronize()
        for b in range(len(good)):
            m0, e0 = o.my_model(good[b])
            np.testing.assert_allclose(model[b].cpu().numpy(), m0, rtol=1e-10, atol=1e-9, err_msg=name)
            np.testing.assert_allclose(err2[b].cpu().numpy(), e0, rtol=1e-14, err_msg=name)
