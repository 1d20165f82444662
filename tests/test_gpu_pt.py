"""GPU parallel-tempering sampler against the oracle sampler.

* replay: with the same Philox stream the FP64 device sampler and the numpy
  oracle (``oracle.pt``) walk the same chain (stretch proposals, Metropolis
  decisions, swaps, ladder adaptation), compared sweep by sweep;
* the graph-captured and the eagerly launched sweep are bit-identical;
* posterior: the mixed-precision sampler on 51 Peg recovers the fit the
  reference recorded (tests/01_51peg_basic.ipynb), and with an independent
  random stream its cold-chain quantiles (51 Peg and the C2 model) agree
  with the oracle sampler's within 4 Monte-Carlo standard errors (batch
  means).
"""
import numpy as np
import pytest
import torch

from astroemperor_gb300 import _native as N
from astroemperor_gb300.engine import PTSampler, default_betas
from oracle.pt import OraclePT
from oracle.rv import OracleRV
from tests.golden.cases import model_51peg

pytestmark = pytest.mark.gpu


def _p0(model, T, W, seed):
    rng = np.random.default_rng(seed)
    lim = model.limits_free()
    lo, hi = lim[:, 0], lim[:, 1]
    # inside the eccentricity support for Ecc_sin/Ecc_cos (|S|,|C| <= 0.7)
    p = rng.uniform(lo, hi, size=(T, W, len(lo)))
    for j, prm in enumerate(model.free_parameters()):
        if prm.name.startswith('Ecc_'):
            p[..., j] *= 0.5
    return p


def _oracle_logpost(o):
    def f(th):
        th = np.atleast_2d(th)
        lp = np.array([o.my_prior(t) for t in th])
        ll = np.array([o.my_likelihood(t) if np.isfinite(x) else -np.inf for t, x in zip(th, lp)])
        return ll, lp
    return f


@pytest.mark.parametrize('adapt', [False, True])
def test_replay_matches_oracle(peg_arr, lib, cuda, adapt):
    m, d = model_51peg(peg_arr, k=1, par=1)
    T, W, S = 4, 16, 12
    betas = np.array([1.0, 0.4, 0.1, 0.01])
    p0 = _p0(m, T, W, 5)
    gpu = PTSampler(W, m.ndim__, m, ntemps=T, betas=betas, precision='fp64', seed=4242,
                    adapt_tau=50, adapt_nu=1, use_graph=False)
    if not adapt:
        gpu.select_adjustment('00')
    gpu.run_mcmc(p0, nsweeps=S)
    o = OracleRV(m.spec(), d.as_dict())
    ora = OraclePT(_oracle_logpost(o), T, W, m.ndim__, betas, adapt=adapt, adapt_tau=50,
                   adapt_nu=1, rng='philox', seed=4242)
    ora.set_positions(p0)
    ora.run(S)
    ch = gpu.get_chain()                        # [T, S, W, D]
    och = np.moveaxis(np.array(ora.chain), 1, 0)
    np.testing.assert_allclose(ch, och, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(gpu.get_log_like(), np.moveaxis(np.array(ora.log_like), 1, 0),
                               rtol=1e-11)
    np.testing.assert_allclose(gpu.get_betas(), np.array(ora.beta_hist), rtol=1e-14)
    np.testing.assert_allclose(gpu.get_tsw(), np.array(ora.tsw_hist), rtol=0, atol=0)
    # mean swap distances are accumulated in FP32 on the device
    np.testing.assert_allclose(gpu.get_smd(), np.array(ora.smd_hist), rtol=1e-5)
    np.testing.assert_allclose(gpu.betas, ora.betas, rtol=1e-14)
    np.testing.assert_array_equal(gpu.accepted, ora.accepted)
    assert ora.accepted.sum() > 0 and np.array(ora.tsw_hist).sum() > 0


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_graph_equals_eager(peg_arr, lib, cuda, precision):
    m, d = model_51peg(peg_arr, k=1, par=1)
    T, W = 3, 32
    p0 = _p0(m, T, W, 9)
    out = []
    for ug in (False, True):
        s = PTSampler(W, m.ndim__, m, ntemps=T, betas=[1.0, 0.3, 0.05], precision=precision,
                      seed=77, use_graph=ug)
        st = s.run_mcmc(p0, nsweeps=25)
        st = s.run_mcmc(st, nsweeps=5)          # continue on the device state
        out.append((s.get_chain(), s.get_log_prob(), s.betas, st.coords))
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)
    assert out[0][0].shape == (T, 30, W, m.ndim__)


def test_posterior_51peg_recovers_reference_fit(peg_arr, lib, cuda):
    """Mixed precision, 51 Peg k=1 parameterisation 1 with the reference
    notebook's conditions; the cold chain must recover the recorded fit."""
    m, d = model_51peg(peg_arr, k=1, par=1)
    m.blocks[0][0].init_pos = [4.1, 4.3]
    m.blocks[0][1].init_pos = [50, 60]
    T, W = 6, 128
    rng = np.random.default_rng(1234)
    lim = m.limits_free()
    p0 = rng.uniform(lim[:, 0], lim[:, 1], size=(T, W, m.ndim__))
    p0[..., 0] = rng.uniform(4.22, 4.24, size=(T, W))
    p0[..., 1] = rng.uniform(50, 60, size=(T, W))
    p0[..., 3:5] *= 0.3
    s = PTSampler(W, m.ndim__, m, ntemps=T, precision='mixed', seed=1)
    s.run_mcmc(p0, nsweeps=3000)
    ch = s.get_chain(flat=True, discard=1500)[0]
    ll = s.get_log_like(flat=True, discard=1500)[0]
    med = np.median(ch, axis=0)
    assert med[0] == pytest.approx(4.2308, abs=5e-4)
    assert med[1] == pytest.approx(55.957, abs=0.8)
    assert med[5] == pytest.approx(3.642, abs=0.6)
    assert med[6] == pytest.approx(2.961, abs=0.8)
    assert ll.max() == pytest.approx(-869.46, abs=0.3)
    assert np.all(np.isfinite(ll))
    lp = s.get_log_prob(flat=True, discard=1500)[0]
    assert np.all(lp <= ll + 1e-9)            # logprior <= 0 for these priors


def test_save_run_round_trip(peg_arr, lib, cuda, tmp_path):
    from astroemperor_gb300.backend_io import load_run
    m, d = model_51peg(peg_arr, k=1, par=1)
    T, W = 3, 16
    s = PTSampler(W, m.ndim__, m, ntemps=T, betas=[1.0, 0.3, 0.05], seed=5)
    s.run_mcmc(_p0(m, T, W, 2), nsweeps=12)
    back = load_run(s.save(str(tmp_path / 'run.h5'), discard=2))
    ch = s.get_chain(discard=2)
    for t in range(T):
        np.testing.assert_array_equal(back[f'mcmc_t{t}/chain'], ch[t])
        np.testing.assert_array_equal(back[f'mcmc_t{t}/accepted'], s.accepted[t])
    np.testing.assert_array_equal(back['mcmc/tsw_history'], s.get_tsw(discard=2))


def test_adaptation_batches_driver_freezes_the_ladder(peg_arr, lib, cuda):
    """support/endit_freeze.scr: adapt in batches, then freeze and sample."""
    m, d = model_51peg(peg_arr, k=1, par=1)
    T, W = 4, 32
    s = PTSampler(W, m.ndim__, m, ntemps=T, betas=[1.0, 0.4, 0.1, 0.01], seed=9, adapt_tau=10)
    state, conv, tau = s.run_adaptation_batches(_p0(m, T, W, 3), adaptation_batches=3,
                                                adaptation_nsweeps=40, nsweeps=30)
    assert s.config_adaptation_halflife == 0
    bh = s.get_betas()
    n = s.iteration
    assert n in (40 + 30, 80 + 30, 120 + 30)
    # adapting before the freeze, constant after it
    assert np.any(bh[n - 31] != bh[0])
    np.testing.assert_array_equal(bh[n - 30:], np.repeat(bh[n - 30:n - 29], 30, axis=0))
    assert np.isfinite(s.get_evidence_ss()[0]) and np.isfinite(s.get_evidence_ti()[0])


def _quantile_se(x_sw, q, nb=10):
    """Monte-Carlo standard error of the q-quantile of a chain x[steps, walkers]
    by batch means: the chain cut into ``nb`` contiguous blocks of sweeps,
    the quantile of each block, their standard deviation over sqrt(nb)
    (valid when a block is much longer than the autocorrelation time; the
    blocks here are 600 sweeps against times of tens to a few hundred)."""
    blocks = np.array_split(x_sw, nb, axis=0)
    bq = np.array([np.quantile(b.reshape(-1), q) for b in blocks])
    return float(np.std(bq, ddof=1) / np.sqrt(nb))


def _compare_quantiles(cpu, gpu, cols, names, nsig=4.0):
    """cpu, gpu: cold chains [steps, walkers, ndim] of independent samplers."""
    for j in cols:
        for q in (0.16, 0.5, 0.84):
            a, b = np.quantile(cpu[:, :, j], q), np.quantile(gpu[:, :, j], q)
            bound = nsig * np.hypot(_quantile_se(cpu[:, :, j], q), _quantile_se(gpu[:, :, j], q))
            print(f'{names[j]} q={q}: oracle {a:.8g} device {b:.8g} |d| {abs(a - b):.3g} bound {bound:.3g}')
            assert abs(a - b) <= bound, (names[j], q, a, b, bound)


def _device_fp64(ctx):
    """Batch log-posterior with the FP64 kernel (equal to the numpy oracle
    to 1e-11 on the golden cases), for the oracle sampler: the numpy path
    would take minutes for these chain lengths."""
    def f(th):
        t = torch.as_tensor(np.atleast_2d(th), dtype=torch.float64, device='cuda:0')
        ll, lp = ctx.logpost(t, precision=N.EMP_PREC_FP64)
        return ll.cpu().numpy(), lp.cpu().numpy()
    return f


def _independent_runs(m, ctx, p0, betas, S, seed_cpu, seed_gpu):
    T, W = p0.shape[:2]
    ora = OraclePT(_device_fp64(ctx), T, W, m.ndim__, betas, adapt=False, rng='numpy', seed=seed_cpu)
    ora.set_positions(p0)
    ora.run(S)
    cpu = np.array(ora.chain)[S // 4:, 0]
    gpu = PTSampler(W, m.ndim__, m, ntemps=T, betas=betas, precision='mixed', seed=seed_gpu, context=ctx)
    gpu.select_adjustment('00')
    gpu.run_mcmc(p0, nsweeps=S)
    return cpu, gpu.get_chain(discard=S // 4)[0]


def test_posterior_quantiles_match_the_oracle_sampler(peg_arr, lib, cuda):
    """Independent random streams (numpy generator in the oracle sampler,
    Philox on the device, mixed precision on the device): the cold-chain
    16/50/84 % quantiles of 51 Peg k=1 agree within 4 Monte-Carlo standard
    errors of their difference."""
    from astroemperor_gb300.engine import Context
    m, d = model_51peg(peg_arr, k=1, par=1)
    ctx = Context(m, 'cuda:0')
    T, W, S = 2, 64, 8000
    rng = np.random.default_rng(11)
    lim = m.limits_free()
    p0 = rng.uniform(lim[:, 0], lim[:, 1], size=(T, W, m.ndim__))
    p0[..., 0] = rng.uniform(4.225, 4.235, size=(T, W))
    p0[..., 1] = rng.uniform(52, 58, size=(T, W))
    p0[..., 3:5] *= 0.3
    cpu, g = _independent_runs(m, ctx, p0, [1.0, 0.2], S, 3, 12345)
    names = [p.name for p in m.free_parameters()]
    _compare_quantiles(cpu, g, (0, 1, 5, 6), names)       # period, amplitude, offset, jitter


def test_posterior_quantiles_match_the_oracle_sampler_c2(lib, cuda):
    """The same check on the two-instrument MA(1) model of the C2 workload
    (3 Keplerians, 23 dimensions)."""
    from astroemperor_gb300 import synth
    from astroemperor_gb300.engine import Context
    m, d, _, truth = synth.build_model('c2', seed=1234)
    ctx = Context(m, 'cuda:0')
    T, W, S = 2, 64, 8000
    rng = np.random.default_rng(5)
    lim = m.limits_free()
    p0 = np.clip(truth + 1e-3 * (lim[:, 1] - lim[:, 0]) * rng.normal(size=(T, W, m.ndim__)),
                 lim[:, 0], lim[:, 1])
    cpu, g = _independent_runs(m, ctx, p0, [1.0, 0.3], S, 17, 99)
    names = [p.name for p in m.free_parameters()]
    cols = [names.index(n) for n in ('Period 1', 'Amplitude 1', 'Amplitude 3', 'Offset 2', 'Jitter 1',
                                     'MACoefficient 1 Order 1')]
    _compare_quantiles(cpu, g, cols, names)


def test_sweep_host_equals_device_sweep(peg_arr, lib, cuda):
    """A sweep through pinned host state (packed and three-tensor forms) is
    the device sweep: same counters and random words, same state after."""
    from astroemperor_gb300.engine import Context, PTState
    m, d = model_51peg(peg_arr, k=1, par=1)
    T, W = 3, 32
    p0 = _p0(m, T, W, 21)
    ctx = Context(m, 'cuda:0')
    ss = [PTSampler(W, m.ndim__, m, ntemps=T, betas=[1.0, 0.3, 0.05], precision='mixed', seed=8,
                    context=ctx, autotune=False) for _ in range(3)]
    for s in ss:
        s.run_mcmc(p0, nsweeps=4)
    h = ss[0].host_state()
    for _ in range(3):
        ss[0].sweep_host_packed(h)
    ht = ss[1].theta.cpu().pin_memory()
    hl = ss[1].logl.cpu().pin_memory()
    hp = ss[1].logprior.cpu().pin_memory()
    for _ in range(3):
        ss[1].sweep_host(ht, hl, hp)
    ss[2].run_mcmc(PTState(ss[2]), nsweeps=3)
    ref = torch.cat([ss[2].theta.reshape(-1), ss[2].logl, ss[2].logprior]).cpu()
    np.testing.assert_array_equal(h.numpy(), ref.numpy())
    np.testing.assert_array_equal(torch.cat([ht.reshape(-1), hl, hp]).numpy(), ref.numpy())
    assert not np.array_equal(ref.numpy()[: T * W * m.ndim__], p0.reshape(-1))
