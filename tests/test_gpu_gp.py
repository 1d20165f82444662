"""Celerite GP likelihood on the device (k_logpost residuals + k_gp) against
the oracle's recursion (which equals the dense Cholesky definition to 1e-14).

Tolerances
  FP64  : |dlogL| / |logL| <= 1e-9 (the device and numpy evaluate the same
          recursion in different operation orders; the GP quadratic form
          amplifies the differences by the conditioning of K)
  mixed : |dlogL| / |logL| <= 1e-6 (residuals from the mixed-precision
          Keplerian pipeline, recursion in FP64)
  PT replay (FP64, same Philox stream): chains within 1e-13, logL 1e-9
The cases include a GP on the residuals of a live MA recurrence (global
MA(1); the documented per-instrument MA(2)), which the kernel forms after the
lane-chunk scan has given each lane its incoming MA state.
"""
import numpy as np
import pytest
import torch

from astroemperor_gb300 import _native as N
from astroemperor_gb300.engine import Context, PTSampler
from oracle.pt import OraclePT
from oracle.rv import OracleRV
from tests.golden.cases import GP_KERNELS, gp_case_models, model_51peg

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-9
MIXED_RTOL = 1e-6


@pytest.fixture(scope='module')
def cases(peg_arr, lib, cuda):
    out = {}
    for name, (m, d, th) in gp_case_models(peg_arr).items():
        o = OracleRV(m.spec(), d.as_dict())
        lp = np.array([o.my_prior(x) for x in th])
        ll = np.array([o.my_likelihood(x) if np.isfinite(p) else -np.inf for x, p in zip(th, lp)])
        out[name] = (m, th, lp, ll, Context(m, 'cuda:0'))
    return out


def _eval(ctx, th, prec):
    t = torch.as_tensor(th, dtype=torch.float64, device='cuda:0')
    ll, lp = ctx.logpost(t, precision=prec)
    torch.cuda.synchronize()
    return ll.cpu().numpy(), lp.cpu().numpy()


@pytest.mark.parametrize('prec', [N.EMP_PREC_FP64, N.EMP_PREC_MIXED])
def test_gp_logpost_matches_oracle(cases, prec):
    tol = FP64_RTOL if prec == N.EMP_PREC_FP64 else MIXED_RTOL
    worst = {}
    for name, (m, th, klp, kll, ctx) in cases.items():
        ll, lp = _eval(ctx, th, prec)
        np.testing.assert_allclose(lp, klp, rtol=1e-13, atol=1e-13, err_msg=name)
        fin = np.isfinite(klp)
        assert np.all(ll[~fin] == -np.inf), name
        assert np.all(np.isfinite(ll[fin])), name
        rel = np.abs(ll[fin] - kll[fin]) / np.abs(kll[fin])
        worst[name] = float(rel.max())
        assert fin.sum() >= 8, name
    print('GP worst relative error per case:', worst)
    assert max(worst.values()) <= tol, worst


def test_gp_logpost_launch_shapes_and_row_counts(cases):
    m, th, klp, kll, ctx = cases['grot']
    ref, _ = _eval(ctx, th, N.EMP_PREC_FP64)
    fin = np.isfinite(ref)
    for L in (8, 32, 128):
        for tile in (0, 64):
            ctx.set_launch(N.EMP_PREC_FP64, L, tile)
            ll, _ = _eval(ctx, th, N.EMP_PREC_FP64)
            np.testing.assert_allclose(ll[fin], ref[fin], rtol=1e-12, err_msg=f'L={L} tile={tile}')
            assert np.all(ll[~fin] == -np.inf)
    ctx.set_launch(N.EMP_PREC_FP64, 0, 0)
    # more rows than before (the row workspace grows), then fewer
    big = np.concatenate([th] * 5)
    ll, _ = _eval(ctx, big, N.EMP_PREC_FP64)
    np.testing.assert_allclose(ll[np.tile(fin, 5)], np.tile(ref[fin], 5), rtol=1e-12)
    ll, _ = _eval(ctx, th[:3], N.EMP_PREC_FP64)
    np.testing.assert_allclose(ll[fin[:3]], ref[:3][fin[:3]], rtol=1e-12)


def _oracle_logpost(o):
    def f(th):
        th = np.atleast_2d(th)
        lp = np.array([o.my_prior(t) for t in th])
        ll = np.array([o.my_likelihood(t) if np.isfinite(x) else -np.inf for t, x in zip(th, lp)])
        return ll, lp
    return f


def _p0_near(m, T, W, seed):
    rng = np.random.default_rng(seed)
    lim = m.limits_free()
    lo, hi = lim[:, 0], lim[:, 1]
    c = np.array([4.231, 55.957, 1.769, 0.087, 0.061, 3.642, 2.961] + [0.0] * (len(lo) - 7))
    c[7:] = 0.3 * (lo[7:] + hi[7:])
    p = c + 0.01 * (hi - lo) * rng.normal(size=(T, W, len(lo)))
    return np.clip(p, lo + 1e-9, hi - 1e-9)


@pytest.mark.parametrize('moav', [None, {'order': 1, 'global': True}])
def test_gp_pt_replay_matches_oracle(peg_arr, lib, cuda, moav):
    """Same Philox stream: the FP64 device sampler (stretch proposals through
    k_logpost, likelihood and Metropolis test in k_gp) walks the oracle's chain;
    with a global MA(1) the GP models the residuals after the recurrence."""
    m, d = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['sho_rho_tau_sigma'], moav=moav, quirk=False)
    T, W, S = 2, 8, 5
    betas = np.array([1.0, 0.2])
    p0 = _p0_near(m, T, W, 3)
    gpu = PTSampler(W, m.ndim__, m, ntemps=T, betas=betas, precision='fp64', seed=99,
                    adapt_tau=50, adapt_nu=1, use_graph=False)
    gpu.select_adjustment('00')
    gpu.run_mcmc(p0, nsweeps=S)
    o = OracleRV(m.spec(), d.as_dict())
    ora = OraclePT(_oracle_logpost(o), T, W, m.ndim__, betas, adapt=False, adapt_tau=50,
                   adapt_nu=1, rng='philox', seed=99)
    ora.set_positions(p0)
    ora.run(S)
    ch = gpu.get_chain()
    och = np.moveaxis(np.array(ora.chain), 1, 0)
    np.testing.assert_allclose(ch, och, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(gpu.get_log_like(), np.moveaxis(np.array(ora.log_like), 1, 0), rtol=FP64_RTOL)
    np.testing.assert_array_equal(gpu.accepted, ora.accepted)
    assert ora.accepted.sum() > 0


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_gp_pt_graph_equals_eager_and_state_consistent(peg_arr, lib, cuda, precision):
    m, d = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['grot'])
    T, W = 3, 16
    p0 = _p0_near(m, T, W, 11)
    out = []
    for ug in (False, True):
        s = PTSampler(W, m.ndim__, m, ntemps=T, betas=[1.0, 0.3, 0.05], precision=precision,
                      seed=5, use_graph=ug)
        st = s.run_mcmc(p0, nsweeps=12)
        out.append((s.get_chain(), s.get_log_like(), s.get_log_prob(), s.betas, st.coords))
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)
    # the stored log-likelihood of every walker is that of its stored theta
    ch, ll = out[0][0], out[0][1]
    o = OracleRV(m.spec(), d.as_dict())
    tol = FP64_RTOL if precision == 'fp64' else MIXED_RTOL
    for t in range(T):
        for w in range(0, W, 5):
            x = ch[t, -1, w]
            ref = o.my_likelihood(x)
            assert abs(ll[t, -1, w] - ref) <= tol * abs(ref), (t, w, ll[t, -1, w], ref)
    assert np.all(np.isfinite(ll[:, -1]))


def test_gp_logl_of_given_residuals(cases):
    """emp_gp_logl on residuals from emp_model_eval equals the GP part of the
    log-posterior entry (FP64) at every theta inside the prior."""
    for name in ('grot', 'real_matern'):
        m, th, klp, kll, ctx = cases[name]
        fin = np.isfinite(klp)
        t = torch.as_tensor(th[fin], dtype=torch.float64, device='cuda:0')
        model, err2 = ctx.model_eval(t)
        y = torch.as_tensor(m.data.RV, dtype=torch.float64, device="cuda:0")
        ll = ctx.gp_logl(t, y[None, :] - model, err2).cpu().numpy()
        ref, _ = _eval(ctx, th[fin], N.EMP_PREC_FP64)
        np.testing.assert_allclose(ll, ref, rtol=1e-12, err_msg=name)
        np.testing.assert_allclose(ll, kll[fin], rtol=FP64_RTOL, err_msg=name)
        # the float-float recursion on the same FP64 residuals
        llf = ctx.gp_logl(t, y[None, :] - model, err2, precision=N.EMP_PREC_MIXED).cpu().numpy()
        np.testing.assert_allclose(llf, ll, rtol=1e-10, err_msg=name)


def test_gp_unsupported_paths(peg_arr, lib, cuda):
    m, d = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['grot'])
    ctx = Context(m, 'cuda:0')
    t = torch.as_tensor(np.tile(m.limits_free().mean(axis=1), (2, 1)), dtype=torch.float64, device='cuda:0')
    with pytest.raises(N.EmpError, match='GP'):
        ctx.logpost_grad(t)
    m0, _ = model_51peg(peg_arr, k=1, par=1)
    ctx0 = Context(m0, 'cuda:0')
    t0 = torch.as_tensor(np.tile(m0.limits_free().mean(axis=1), (2, 1)), dtype=torch.float64, device='cuda:0')
    r = torch.zeros(2, m0.data.ndata, dtype=torch.float64, device='cuda:0')
    with pytest.raises(N.EmpError, match='no GP'):
        ctx0.gp_logl(t0, r, r + 1.0)
    # a batch handle takes GP models, but not the residual-row entry
    from astroemperor_gb300.batch import BatchContext
    bctx = BatchContext([m, m], 'cuda:0')
    rb = torch.zeros(2, m.data.ndata, dtype=torch.float64, device='cuda:0')
    out = torch.empty(2, dtype=torch.float64, device='cuda:0')
    with pytest.raises(N.EmpError, match='one-system'):
        N.call('emp_gp_logl', bctx.h, t.data_ptr(), 2, rb.data_ptr(), (rb + 1.0).data_ptr(), out.data_ptr(),
               int(N.EMP_PREC_FP64), None)


def test_gp_with_quirk_moav_on_device(peg_arr, lib, cuda):
    """The reference's per-instrument MOAV is a no-op; with the quirk a GP model
    carrying it evaluates like the same model without it."""
    m0, d = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['grot'])
    mq, _ = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['grot'], moav={'order': 1, 'global': False},
                        quirk=True)
    rng = np.random.default_rng(3)
    th0 = _p0_near(m0, 1, 12, 4)[0]
    thq = np.concatenate([th0[:, :7], np.tile([0.1, 10.0], (12, 1)), th0[:, 7:]], axis=1)
    for prec in (N.EMP_PREC_FP64, N.EMP_PREC_MIXED):
        a, _ = _eval(Context(m0, 'cuda:0'), th0, prec)
        b, _ = _eval(Context(mq, 'cuda:0'), thq, prec)
        np.testing.assert_allclose(b, a, rtol=1e-12)
    o = OracleRV(mq.spec(), d.as_dict())
    ref = np.array([o.my_likelihood(x) for x in thq])
    a, _ = _eval(Context(mq, 'cuda:0'), thq, N.EMP_PREC_FP64)
    np.testing.assert_allclose(a, ref, rtol=FP64_RTOL)
