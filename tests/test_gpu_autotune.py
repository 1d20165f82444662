"""Autotuner: every candidate shape gives the same log-posterior; the chosen
shape is at least as fast as the library default on the same batch."""
import numpy as np
import pytest
import torch

from astroemperor_gb300 import _native as N
from astroemperor_gb300 import autotune as at
from astroemperor_gb300 import synth
from astroemperor_gb300.engine import Context

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_fast_correct_shape(lib, cuda):
    model, data, setup, truth = synth.build_model('c2', seed=5)
    ctx = Context(model, 'cuda:0')
    th = at.representative_batch(model, 1280, 'cuda:0')
    ctx.set_launch(N.EMP_PREC_MIXED, 0, 0)
    ref_ll, _ = ctx.logpost(th, precision=N.EMP_PREC_MIXED)
    s = torch.cuda.Stream()
    t_default = at.time_launch(ctx, th, N.EMP_PREC_MIXED, 5, s)
    L, tile, ms = at.autotune(ctx, th, N.EMP_PREC_MIXED, use_cache=False)
    assert ctx.get_launch(N.EMP_PREC_MIXED) == (L, tile)
    t_tuned = at.time_launch(ctx, th, N.EMP_PREC_MIXED, 5, s)
    assert t_tuned <= 1.15 * t_default, (t_tuned, t_default)
    ll, _ = ctx.logpost(th, precision=N.EMP_PREC_MIXED)
    torch.cuda.synchronize()
    a, b = ll.cpu().numpy(), ref_ll.cpu().numpy()
    fin = np.isfinite(b)
    np.testing.assert_allclose(a[fin], b[fin], rtol=2e-7)
    assert np.all(a[~fin] == -np.inf)
