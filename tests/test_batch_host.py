"""Host side of the ragged batch: the seeded system generator and the
per-system Philox key."""
import numpy as np

from astroemperor_gb300 import synth
from astroemperor_gb300.batch import GOLDEN, pad_rows, system_seed


def test_ragged_systems_are_reproducible_and_in_range():
    a = synth.make_ragged(12, seed=5)
    b = synth.make_ragged(12, seed=5)
    for (ma, da, ta), (mb, db, tb) in zip(a, b):
        np.testing.assert_array_equal(da.BJD, db.BJD)
        np.testing.assert_array_equal(da.RV, db.RV)
        np.testing.assert_array_equal(ta, tb)
        assert ma.ndim__ == mb.ndim__
    cfg = synth.RAGGED
    for m, d, th in a:
        assert cfg['n_range'][0] <= d.ndata <= cfg['n_range'][1]
        assert 1 <= d.nins <= 3
        kp = sum(1 for blk in m.blocks if blk.type_ == 'Keplerian')
        assert 1 <= kp <= 4
        assert m.ndim__ == 5 * kp + 2 * d.nins
        assert d.BJD.max() <= cfg['span'][1]
    # any subset regenerates identically (per-system generators)
    m5, d5, _ = synth.ragged_model(5, 7)
    np.testing.assert_array_equal(d5.RV, a[7][1].RV)


def test_system_seed_and_padding():
    assert system_seed(0, 0) == 0
    assert system_seed(1, 1) == (1 + GOLDEN) % 2 ** 64
    assert system_seed(2 ** 64 - 1, 2) == (2 ** 64 - 1 + 2 * GOLDEN) % 2 ** 64
    p = pad_rows([np.ones((2, 3)), 2 * np.ones((2, 5))], 6)
    assert p.shape == (2, 2, 6)
    assert p[0, :, 3:].sum() == 0 and p[1, :, :5].sum() == 20
