"""emp_pt_sweep_static: the PT sweep for callers that cannot allocate.

Some callers of this library cannot call cudaMalloc: code that runs while a
larger application graph is being captured, or a host program whose device
memory is one fixed arena owned by its own allocator.  For them
emp_pt_sweep_static runs the same sweep as emp_pt_sweep with its workspace
in a static device array of the library instead of a caller buffer.

This test drives two identical samplers, one through emp_pt_sweep (caller
workspace) and one through emp_pt_sweep_static, for two sweeps in a row
through the C ABI, and requires the same chains, log-likelihoods, ladder,
swap rates and positions (the swap distances are FP32 sums of atomics, so
they agree to rtol 1e-5).  It also checks the size limit.  It builds its own
model so it runs alone in a fresh process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from astroemperor_gb300 import _native as N
from astroemperor_gb300.engine import PTSampler
from tests.golden.cases import model_51peg

pytestmark = pytest.mark.gpu


def _sampler(m, p0, seed):
    s = PTSampler(16, m.ndim__, m, ntemps=4, betas=[1.0, 0.5, 0.2, 0.05], precision='fp64',
                  seed=seed, use_graph=False)
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


def test_static_workspace_sweep_matches_caller_workspace(peg_arr, lib, cuda):
    m, d = model_51peg(peg_arr, k=1, par=1)
    rng = np.random.default_rng(11)
    lim = m.limits_free()
    p0 = rng.uniform(lim[:, 0], lim[:, 1], size=(4, 16, m.ndim__))
    p0[..., 3:5] *= 0.5
    a = _sampler(m, p0, 99)
    b = _sampler(m, p0, 99)
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
