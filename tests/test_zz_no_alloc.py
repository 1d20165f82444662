"""emp_pt_sweep_static: the PT sweep for callers that cannot allocate.

Some callers of this library cannot call cudaMalloc: a host program whose
device memory is one fixed arena owned by its own allocator, or a process
that allows no allocation once it runs.  For them emp_pt_sweep_static runs
the same sweep as emp_pt_sweep with its workspace in a static device array
of the library instead of a caller buffer.

These tests drive two identical samplers, one through emp_pt_sweep (caller
workspace) and one through emp_pt_sweep_static, for two sweeps in a row
through the C ABI, in FP64 and mixed precision on one system and on a
two-system batch handle (whose persistent launch takes its item counter
from the workspace), and require the same chains, log-likelihoods, ladder,
swap rates and positions (the swap distances are FP32 sums of atomics, so
they agree to rtol 1e-5).  They also check the size limit.  They build their
own models, so they run alone in a fresh process as well as after the other
tests.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from astroemperor_gb300 import _native as N
from astroemperor_gb300.engine import PTSampler
from tests.golden.cases import model_51peg

pytestmark = pytest.mark.gpu


def _sampler(m, p0, seed, precision='fp64'):
    s = PTSampler(16, m.ndim__, m, ntemps=4, betas=[1.0, 0.5, 0.2, 0.05], precision=precision,
                  seed=seed, use_graph=False, autotune=False)
    s.set_positions(p0)
    s._grow(4)
    torch.cuda.synchronize()
    return s


def _hist(s):
    n = int(s.n_rec[0].item())
    return dict(chain=s.chain[:n].cpu().numpy(), ll=s.log_like_h[:n].cpu().numpy(),
                lp=s.log_prob_h[:n].cpu().numpy(), beta=s.beta_h[:n].cpu().numpy(),
                tsw=s.tsw_h[:n].cpu().numpy(), smd=s.smd_h[:n].cpu().numpy(),
                theta=s.theta.cpu().numpy(), members=s.members.cpu().numpy(),
                betas=s.betas_d.cpu().numpy(), accepted=s.accepted_d.cpu().numpy())


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_static_workspace_sweep_matches_caller_workspace(peg_arr, lib, cuda, precision):
    m, d = model_51peg(peg_arr, k=1, par=1)
    rng = np.random.default_rng(11)
    lim = m.limits_free()
    p0 = rng.uniform(lim[:, 0], lim[:, 1], size=(4, 16, m.ndim__))
    p0[..., 3:5] *= 0.5
    a = _sampler(m, p0, 99, precision)
    b = _sampler(m, p0, 99, precision)
    for _ in range(2):                                    # two calls in a row
        sa, ra = a._state_struct(1), a._record_struct()
        N.call('emp_pt_sweep', a.ctx.h, C.byref(sa), C.byref(ra), a.stream.cuda_stream)
        sb, rb = b._state_struct(1), b._record_struct()
        sb.work, sb.work_bytes = None, 0                  # no caller workspace at all
        N.call('emp_pt_sweep_static', b.ctx.h, C.byref(sb), C.byref(rb), b.stream.cuda_stream)
        torch.cuda.synchronize()
    ha, hb = _hist(a), _hist(b)
    assert ha['chain'].shape[0] == 2
    for k in ('chain', 'll', 'lp', 'beta', 'tsw', 'theta', 'members', 'betas', 'accepted'):
        np.testing.assert_array_equal(ha[k], hb[k], err_msg=k)
    np.testing.assert_allclose(ha['smd'], hb['smd'], rtol=1e-5)
    assert ha['tsw'].sum() > 0


def test_static_workspace_rejects_too_many_walkers(peg_arr, lib, cuda):
    m, d = model_51peg(peg_arr, k=1, par=1)
    s = PTSampler(16, m.ndim__, m, ntemps=2, betas=[1.0, 0.5], precision='fp64', seed=1)
    st = s._state_struct(1)
    st.ntemps, st.nwalkers = 256, 256                     # 65536 walkers > 32768
    rc = s.ctx.lib.emp_pt_sweep_static(s.ctx.h, C.byref(st), None, None)
    assert rc == N.EMP_E_SIZE
    assert b'static workspace' in s.ctx.lib.emp_last_error_string()


def test_static_workspace_batch_matches_caller_workspace(lib, cuda):
    """Two systems of the ragged survey on one batch handle."""
    from astroemperor_gb300 import synth
    from astroemperor_gb300.batch import BatchContext, BatchPTSampler
    systems = [synth.ragged_model(7, s) for s in (3, 11)]
    models = [m for m, d, t in systems]
    ctx = BatchContext(models, 'cuda:0')
    T, W = 3, 16
    rng = np.random.default_rng(4)
    p0 = []
    for m, d, truth in systems:
        lim = m.limits_free()
        p0.append(np.clip(truth + 1e-3 * (lim[:, 1] - lim[:, 0]) * rng.normal(size=(T, W, m.ndim__)),
                          lim[:, 0], lim[:, 1]))
    p0 = ctx.pad(p0)
    samplers = []
    for _ in range(2):
        s = BatchPTSampler(ctx, ntemps=T, nwalkers=W, betas=[1.0, 0.4, 0.1], precision='mixed', seed=5,
                           use_graph=False, autotune=False)
        s.set_positions(p0)
        s._grow(4)
        samplers.append(s)
    torch.cuda.synchronize()
    a, b = samplers
    for _ in range(2):                                    # two calls in a row
        sa, ra = a._state_struct(1), a._record_struct()
        N.call('emp_pt_sweep', ctx.h, C.byref(sa), C.byref(ra), a.stream.cuda_stream)
        sb, rb = b._state_struct(1), b._record_struct()
        sb.work, sb.work_bytes = None, 0
        N.call('emp_pt_sweep_static', ctx.h, C.byref(sb), C.byref(rb), b.stream.cuda_stream)
        torch.cuda.synchronize()
    assert int(a.n_rec[0].item()) == int(b.n_rec[0].item()) == 2
    for name in ('chain', 'log_like_h', 'log_prob_h', 'beta_h', 'tsw_h', 'theta', 'logl', 'members',
                 'betas_d', 'accepted_d'):
        np.testing.assert_array_equal(getattr(a, name).cpu().numpy(), getattr(b, name).cpu().numpy(),
                                      err_msg=name)
    assert not np.array_equal(a.theta.cpu().numpy(), p0.reshape(-1, ctx.ndim))
