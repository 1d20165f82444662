"""Joint RV + astrometry models on a batch handle (emp_create_batch with one
astrometry descriptor per system, emp_set_astrometry).

* batch log-posterior rows of the HIP 21850 model and its two-planet variant
  equal their one-system handles bit for bit, in both precisions, and the
  long-double values of the fixtures (FP64 5e-10, mixed 1e-6 relative);
* a batched PT run equals one-system runs keyed seed + s * 0x9E3779B97F4A7C15
  with the same launch shape, bit for bit (positions, logL, ladders,
  acceptance counts, chains and histories), in both precisions.
"""
import os

import numpy as np
import pytest
import torch

from astroemperor_gb300 import _native as N
from astroemperor_gb300.batch import BatchContext, BatchPTSampler, system_seed
from astroemperor_gb300.engine import Context, PTSampler
from tests.golden.cases import HIP_K2_PLANET, HIP_MAP, model_hip21850
from tests.test_gpu_batch import _compare_system

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
LAUNCH = (16, 512)


def _systems():
    fix = np.load(os.path.join(GOLDEN, 'hip21850.npz'))
    kat = np.load(os.path.join(GOLDEN, 'am_kat.npz'))
    out = []
    for planets, pre in ((1, ''), (2, 'k2__'), (1, '')):
        model, data, am = model_hip21850(fix, planets)
        out.append((model, kat[f'{pre}theta'], kat[f'{pre}logl_ld'], kat[f'{pre}logprior']))
    return out


@pytest.mark.parametrize('prec,tol', [(N.EMP_PREC_FP64, 5e-10), (N.EMP_PREC_MIXED, 1e-6)])
def test_am_batch_logpost_matches_single(lib, cuda, prec, tol):
    sy = _systems()
    models = [m for m, _, _, _ in sy]
    bctx = BatchContext(models)
    bctx.set_launch(prec, *LAUNCH)
    rows = [th for _, th, _, _ in sy]
    assert len({len(r) for r in rows}) == 1
    ll, lp = bctx.logpost(torch.as_tensor(bctx.pad(rows), device='cuda:0'), precision=prec)
    ll, lp = ll.cpu().numpy(), lp.cpu().numpy()
    for s, (m, th, ld, klp) in enumerate(sy):
        ctx = Context(m, 'cuda:0')
        ctx.set_launch(prec, *LAUNCH)
        l1, p1 = ctx.logpost(torch.as_tensor(th, device='cuda:0'), precision=prec)
        np.testing.assert_array_equal(ll[s], l1.cpu().numpy(), err_msg=f'system {s}')
        np.testing.assert_array_equal(lp[s], p1.cpu().numpy(), err_msg=f'system {s}')
        np.testing.assert_allclose(lp[s], klp, rtol=1e-13, atol=1e-13)
        fin = np.isfinite(klp)
        assert fin.sum() >= 8 and np.all(ll[s][~fin] == -np.inf)
        assert np.max(np.abs(ll[s][fin] - ld[fin]) / np.abs(ld[fin])) <= tol


@pytest.mark.parametrize('prec', ['fp64', 'mixed'])
def test_am_batch_pt_equals_single_system_runs(lib, cuda, prec):
    sy = _systems()
    models = [m for m, _, _, _ in sy]
    T, W, sweeps, seed = 3, 16, 12, 31
    betas = [1.0, 0.3, 0.05]
    rng = np.random.default_rng(9)
    p0 = []
    for m in models:
        lim = m.limits_free()
        c = np.array(HIP_MAP if m.ndim__ == len(HIP_MAP) else HIP_MAP[:7] + HIP_K2_PLANET + HIP_MAP[7:])
        p0.append(np.clip(c + 1e-3 * (lim[:, 1] - lim[:, 0]) * rng.normal(size=(T, W, len(c))),
                          lim[:, 0], lim[:, 1]))
    pcode = N.EMP_PREC_FP64 if prec == 'fp64' else N.EMP_PREC_MIXED
    bctx = BatchContext(models)
    bctx.set_launch(pcode, *LAUNCH)
    bt = BatchPTSampler(bctx, ntemps=T, nwalkers=W, betas=betas, adapt_tau=20, precision=prec,
                        seed=seed, autotune=False)
    bt.run(bctx.pad(p0), nsweeps=sweeps)
    for s, m in enumerate(models):
        ctx = Context(m, 'cuda:0')
        ctx.set_launch(pcode, *LAUNCH)
        single = PTSampler(W, m.ndim__, m, ntemps=T, betas=betas, adapt_tau=20, precision=prec,
                           seed=system_seed(seed, s), context=ctx, autotune=False, smd_history=False)
        single.run_mcmc(p0[s], nsweeps=sweeps)
        _compare_system(bt, s, single)
    assert bt.accepted.sum() > 0 and bt.swaps_accepted.sum() > 0
