"""Ragged batch of independent systems (one handle, one sweep sequence).

* batch log-posterior rows equal the one-system handle's, bit for bit, and
  the FP64 oracle within the precision's tolerance (FP64 1e-11, mixed 1e-6
  relative);
* a batched PT run equals S one-system runs keyed seed + s * 0x9E3779B97F4A7C15
  with the same launch shape: positions, logL, ladders, acceptance counts,
  cold chains and histories, bit for bit;
* at the full ragged size (4096 systems, 8 x 64 walkers) the stored logL of
  every walker equals a fresh evaluation of its position, and sampled
  systems equal their one-system runs.
"""
import numpy as np
import pytest
import torch

from astroemperor_gb300 import _native as N
from astroemperor_gb300 import synth
from astroemperor_gb300.batch import BatchContext, BatchPTSampler, pad_rows, system_seed
from astroemperor_gb300.engine import Context, PTSampler
from oracle.rv import OracleRV

pytestmark = pytest.mark.gpu

LAUNCH = (16, 512)


def _near_truth(model, truth, shape, rng, scale=1e-3):
    lim = model.limits_free()
    lo, hi = lim[:, 0], lim[:, 1]
    c = np.clip(truth, lo, hi)
    p = c + scale * (hi - lo) * rng.normal(size=shape + (len(lo),))
    return np.clip(p, lo, hi)


def _systems(n, seed=7):
    return synth.make_ragged(n, seed=seed)


@pytest.mark.parametrize('prec,tol', [(N.EMP_PREC_FP64, 1e-11), (N.EMP_PREC_MIXED, 1e-6)])
def test_batch_logpost_matches_single_and_oracle(lib, cuda, prec, tol):
    sy = _systems(6)
    models = [m for m, _, _ in sy]
    bctx = BatchContext(models)
    bctx.set_launch(prec, *LAUNCH)
    rng = np.random.default_rng(1)
    B = 24
    rows = [_near_truth(m, th, (B,), rng, scale=0.05) for m, _, th in sy]
    theta = torch.as_tensor(bctx.pad(rows), device='cuda:0')
    ll, lp = bctx.logpost(theta, precision=prec)
    ll, lp = ll.cpu().numpy(), lp.cpu().numpy()
    for s, (m, d, _) in enumerate(sy):
        ctx = Context(m)
        ctx.set_launch(prec, *LAUNCH)
        l1, p1 = ctx.logpost(torch.as_tensor(rows[s], device='cuda:0'), precision=prec)
        np.testing.assert_array_equal(ll[s], l1.cpu().numpy())
        np.testing.assert_array_equal(lp[s], p1.cpu().numpy())
        o = OracleRV(m.spec(), d.as_dict())
        want_lp = np.array([o.my_prior(x) for x in rows[s]])
        np.testing.assert_allclose(lp[s], want_lp, rtol=1e-13, atol=1e-13)
        ok = np.isfinite(want_lp)
        want_ll = np.array([o.my_likelihood(x) for x in rows[s][ok]])
        assert np.max(np.abs(ll[s][ok] - want_ll) / np.abs(want_ll)) <= tol


def _compare_system(bt, s, single):
    T, W = bt.ntemps, bt.nwalkers
    np.testing.assert_array_equal(bt.coords(s), single._coords_host())
    np.testing.assert_array_equal(bt.log_like()[s], single._logl_host())
    np.testing.assert_array_equal(bt.betas[s], single.betas)
    np.testing.assert_array_equal(bt.accepted[s], single.accepted)
    np.testing.assert_array_equal(bt.swaps_accepted[s], single.swaps_d.cpu().numpy())
    # cold chain and histories
    np.testing.assert_array_equal(bt.get_chain(s), single.get_chain()[0])
    np.testing.assert_array_equal(bt.get_log_like(s), single.get_log_like()[0])
    np.testing.assert_array_equal(bt.get_log_prob(s), single.get_log_prob()[0])
    np.testing.assert_array_equal(bt.get_betas(s), single.get_betas())
    if T > 1:
        np.testing.assert_array_equal(bt.get_tsw(s), single.get_tsw())


@pytest.mark.parametrize('prec', ['fp64', 'mixed'])
def test_batch_pt_equals_single_system_runs(lib, cuda, prec):
    sy = _systems(5, seed=3)
    models = [m for m, _, _ in sy]
    T, W, sweeps, seed = 4, 16, 25, 99
    rng = np.random.default_rng(2)
    p0 = [_near_truth(m, th, (T, W), rng) for m, _, th in sy]
    bctx = BatchContext(models)
    pcode = N.EMP_PREC_FP64 if prec == 'fp64' else N.EMP_PREC_MIXED
    bctx.set_launch(pcode, *LAUNCH)
    bt = BatchPTSampler(bctx, ntemps=T, nwalkers=W, betas=[1.0, 0.5, 0.2, 0.05], adapt_tau=20,
                        precision=prec, seed=seed, autotune=False)
    bt.run(bctx.pad(p0), nsweeps=sweeps)
    assert bt.iteration == sweeps
    for s, m in enumerate(models):
        ctx = Context(m)
        ctx.set_launch(pcode, *LAUNCH)
        single = PTSampler(W, m.ndim__, m, ntemps=T, betas=[1.0, 0.5, 0.2, 0.05], adapt_tau=20,
                           precision=prec, seed=system_seed(seed, s), context=ctx, autotune=False,
                           smd_history=False)
        single.run_mcmc(p0[s], nsweeps=sweeps)
        _compare_system(bt, s, single)
    assert bt.accepted.sum() > 0 and bt.swaps_accepted.sum() > 0


def test_batch_graph_equals_eager(lib, cuda):
    sy = _systems(4, seed=5)
    models = [m for m, _, _ in sy]
    T, W = 3, 8
    rng = np.random.default_rng(4)
    p0 = pad_rows([_near_truth(m, th, (T, W), rng) for m, _, th in sy], max(m.ndim__ for m in models))
    out = []
    for graph in (True, False):
        bctx = BatchContext(models)
        bctx.set_launch(N.EMP_PREC_MIXED, *LAUNCH)
        bt = BatchPTSampler(bctx, ntemps=T, nwalkers=W, seed=11, use_graph=graph, autotune=False)
        bt.run(p0, nsweeps=10)
        out.append((bt.coords(), bt.log_like(), bt.betas, bt.get_chain(2)))
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


def test_c3_full_size_consistency(lib, cuda):
    """4096 ragged systems, 8 temperatures x 64 walkers, autotuned shape."""
    sy = synth.make_ragged()
    models = [m for m, _, _ in sy]
    T, W, sweeps, seed = 8, 64, 4, 2024
    rng = np.random.default_rng(9)
    bctx = BatchContext(models)
    p0 = bctx.pad([_near_truth(m, th, (T, W), rng) for m, _, th in sy])
    bt = BatchPTSampler(bctx, ntemps=T, nwalkers=W, seed=seed, record=True)
    bt.run(p0, nsweeps=sweeps)
    L, tile, _ = bt.launch
    # stored logL of every walker == a fresh evaluation of its position
    pos = torch.as_tensor(bt.coords().reshape(bt.S, T * W, bt.ndim), device='cuda:0')
    ll, lp = bctx.logpost(pos, precision=N.EMP_PREC_MIXED)
    np.testing.assert_array_equal(ll.cpu().numpy().reshape(bt.S, T, W), bt.log_like())
    np.testing.assert_array_equal(lp.cpu().numpy().reshape(bt.S, T, W), bt.log_prior())
    assert np.isfinite(bt.log_like()).all()
    assert bt.accepted.sum() > 0
    # sampled systems against their one-system runs (same shape)
    for s in (0, 1, 777, 4095):
        m = models[s]
        ctx = Context(m)
        ctx.set_launch(N.EMP_PREC_MIXED, L, tile)
        single = PTSampler(W, m.ndim__, m, ntemps=T, seed=system_seed(seed, s), context=ctx,
                           autotune=False, smd_history=False)
        single.run_mcmc(p0[s, :, :, : m.ndim__], nsweeps=sweeps)
        _compare_system(bt, s, single)
