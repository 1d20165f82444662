"""Celerite GP likelihoods on a batch handle (emp_create_batch).

A batch runs every system's GP with one state dimension M, the largest of
its systems (a power of two); a system with fewer dimensions leaves the rest
zero, and a system without GP terms gets the Gaussian likelihood from the
same recursion (D_n = err2_n, W_n = 0).

* log-posterior rows of a ragged GP batch (GonzRotation on 256 epochs,
  Rotation on 128, SHO on 226, no GP on 120, Real + Matern32 on 86):
  systems whose own M equals the batch's equal their one-system
  handles bit for bit; the others within 1e-12 (FP64) / 1e-9 (mixed) of
  them, the system without GP terms within 1e-12 / 1e-6 (its one-system
  handle sums the Gaussian terms in another pipeline); every row within
  the GP tolerances of the oracle (FP64 1e-9, mixed 1e-6 relative);
* the same with a live global MA(1) under every GP;
* a batched PT run equals one-system runs keyed seed + s * 0x9E3779B97F4A7C15
  with the same launch shape, bit for bit (positions, logL, ladders,
  acceptance counts, chains and histories), in both precisions.
"""
import numpy as np
import pytest
import torch

from astroemperor_gb300 import _native as N
from astroemperor_gb300.batch import BatchContext, BatchPTSampler, system_seed
from astroemperor_gb300.engine import Context, PTSampler
from oracle.rv import OracleRV
from tests.golden.cases import GP_KERNELS, PEG_MAP_P1, draw_thetas, model_51peg
from tests.test_gpu_batch import _compare_system, _near_truth

pytestmark = pytest.mark.gpu

LAUNCH = (16, 512)
FP64_RTOL = 1e-9
MIXED_RTOL = 1e-6


def _centre(m):
    """The 51 Peg fit, GP hyperparameters at the middle of their limits."""
    lim = m.limits_free()
    c = np.array(PEG_MAP_P1 + [0.0] * (len(lim) - len(PEG_MAP_P1)))
    for j in range(len(PEG_MAP_P1), len(lim)):
        c[j] = 0.5 * (lim[j, 0] + lim[j, 1])
    return np.clip(c, lim[:, 0], lim[:, 1])


def _systems(arr, kinds, moav=None):
    """(model, data, own state dimension) per (epoch subset, GP kernel name or None)."""
    out = []
    for rows, kind in kinds:
        m, d = model_51peg(arr[rows], k=1, par=1, gp=GP_KERNELS[kind] if kind else None,
                           moav=moav, quirk=False)
        dims = {'grot': 4, 'rotation': 4, 'real_matern': 3, 'sho_rho_tau_sigma': 2, None: 0}[kind]
        out.append((m, d, 1 << max(1, int(np.ceil(np.log2(max(dims, 1))))) if dims else 0))
    return out


RAGGED = [(slice(None), 'grot'), (slice(None, None, 2), 'rotation'), (slice(30, None), 'sho_rho_tau_sigma'),
          (slice(None, 120), None), (slice(None, None, 3), 'real_matern')]


def _thetas(sy, rng):
    th = [draw_thetas(m, rng, n_in=12, center=_centre(m), n_near=8) for m, _, _ in sy]
    assert len({len(t) for t in th}) == 1
    return th


def _check_logpost(sy, prec, rng):
    models = [m for m, _, _ in sy]
    bctx = BatchContext(models)
    bctx.set_launch(prec, *LAUNCH)
    rows = _thetas(sy, rng)
    theta = torch.as_tensor(bctx.pad(rows), device='cuda:0')
    ll, lp = bctx.logpost(theta, precision=prec)
    ll, lp = ll.cpu().numpy(), lp.cpu().numpy()
    M = max(own for _, _, own in sy)
    tol = FP64_RTOL if prec == N.EMP_PREC_FP64 else MIXED_RTOL
    worst = 0.0
    for s, (m, d, own) in enumerate(sy):
        ctx = Context(m)
        ctx.set_launch(prec, *LAUNCH)
        l1, p1 = ctx.logpost(torch.as_tensor(rows[s], device='cuda:0'), precision=prec)
        l1, p1 = l1.cpu().numpy(), p1.cpu().numpy()
        np.testing.assert_array_equal(lp[s], p1)
        fin = np.isfinite(p1)
        assert fin.sum() >= 8
        np.testing.assert_array_equal(ll[s][~fin], l1[~fin])
        if own == M:
            np.testing.assert_array_equal(ll[s], l1, err_msg=f'system {s}')
        elif own > 0:
            np.testing.assert_allclose(ll[s][fin], l1[fin], rtol=1e-12 if prec == N.EMP_PREC_FP64 else 1e-9,
                                       err_msg=f'system {s}')
        else:
            # no GP terms: the batch forms this system's Gaussian likelihood
            # through the recursion, the one-system handle through its own
            # sum (in the mixed precision: float-float recursion on FP32
            # residuals against the compensated FP32 pipeline)
            np.testing.assert_allclose(ll[s][fin], l1[fin], rtol=1e-12 if prec == N.EMP_PREC_FP64 else tol,
                                       err_msg=f'system {s}')
        o = OracleRV(m.spec(), d.as_dict())
        want = np.array([o.my_likelihood(x) for x in rows[s][fin]])
        rel = np.max(np.abs(ll[s][fin] - want) / np.abs(want))
        worst = max(worst, rel)
        assert rel <= tol, (s, rel)
    print(f'GP batch of {len(sy)} systems ({"FP64" if prec == N.EMP_PREC_FP64 else "mixed"}): '
          f'max relative logL error against the oracle {worst:.2e}')


@pytest.mark.parametrize('prec', [N.EMP_PREC_FP64, N.EMP_PREC_MIXED])
def test_gp_batch_logpost_matches_single_and_oracle(peg_arr, lib, cuda, prec):
    _check_logpost(_systems(peg_arr, RAGGED), prec, np.random.default_rng(31))


@pytest.mark.parametrize('prec', [N.EMP_PREC_FP64, N.EMP_PREC_MIXED])
def test_gp_batch_with_global_ma(peg_arr, lib, cuda, prec):
    sy = _systems(peg_arr, [(slice(None), 'grot'), (slice(None, None, 2), 'rotation'),
                            (slice(20, 200), 'sho_rho_tau_sigma')],
                  moav={'order': 1, 'global': True})
    _check_logpost(sy, prec, np.random.default_rng(32))


@pytest.mark.parametrize('prec', ['fp64', 'mixed'])
def test_gp_batch_pt_equals_single_system_runs(peg_arr, lib, cuda, prec):
    sy = _systems(peg_arr, [(slice(None), 'grot'), (slice(None, None, 2), 'rotation'),
                            (slice(40, None), 'real_matern')])
    models = [m for m, _, _ in sy]
    T, W, sweeps, seed = 3, 16, 20, 77
    betas = [1.0, 0.4, 0.1]
    rng = np.random.default_rng(5)
    p0 = [_near_truth(m, _centre(m), (T, W), rng) for m in models]
    pcode = N.EMP_PREC_FP64 if prec == 'fp64' else N.EMP_PREC_MIXED
    bctx = BatchContext(models)
    bctx.set_launch(pcode, *LAUNCH)
    bt = BatchPTSampler(bctx, ntemps=T, nwalkers=W, betas=betas, adapt_tau=20, precision=prec,
                        seed=seed, autotune=False)
    bt.run(bctx.pad(p0), nsweeps=sweeps)
    assert bt.iteration == sweeps
    for s, m in enumerate(models):
        ctx = Context(m)
        ctx.set_launch(pcode, *LAUNCH)
        single = PTSampler(W, m.ndim__, m, ntemps=T, betas=betas, adapt_tau=20, precision=prec,
                           seed=system_seed(seed, s), context=ctx, autotune=False, smd_history=False)
        single.run_mcmc(p0[s], nsweeps=sweeps)
        _compare_system(bt, s, single)
    assert bt.accepted.sum() > 0 and bt.swaps_accepted.sum() > 0
    # every stored logL is the likelihood of its stored position
    for s, (m, d, _) in enumerate(sy):
        o = OracleRV(m.spec(), d.as_dict())
        xs = bt.coords(s).reshape(-1, m.ndim__)
        want = np.array([o.my_likelihood(x) for x in xs[:8]])
        got = bt.log_like()[s].reshape(-1)[:8]
        tol = FP64_RTOL if prec == 'fp64' else MIXED_RTOL
        assert np.max(np.abs(got - want) / np.abs(want)) <= tol
