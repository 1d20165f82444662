"""Hill stability prior: the oracle's restatement against the reference's own
support/priors/Hill.prior (executed from the reference's files by
tests/golden/make_golden.py into hill_kat.npz), and its compilation into the
model descriptor."""
import numpy as np

from astroemperor_gb300 import _native as N
from oracle.rv import OracleRV, prior_Hill
from tests.golden.cases import model_51peg


def test_oracle_hill_equals_reference_fixture():
    h = np.load('tests/golden/hill_kat.npz')
    got = np.array([prior_Hill(x[:, :int(a[0])], None, [int(a[0]), a[1]]) for x, a in zip(h['x'], h['args'])])
    np.testing.assert_array_equal(got, h['value'])
    assert 0 < np.isfinite(got).sum() < len(got)


def test_hill_keeps_gamma_in_input_order():
    # the reference sorts axes and masses but not gamma = sqrt(1 - e): with
    # the eccentric planet listed first the outcome differs from a version
    # that sorts gamma too
    per = np.array([2.3, 35.0])
    amp = np.array([12.4, 1.1])
    ecc = np.array([0.58, 0.01])
    got = prior_Hill(np.array([per, amp, ecc]), None, [2, 1.0])
    swapped = prior_Hill(np.array([per[::-1], amp[::-1], ecc[::-1]]), None, [2, 1.0])
    assert got == -np.inf and swapped == 0.0


def test_descriptor_hill_mask(peg_arr):
    m, _ = model_51peg(peg_arr, k=3, par=0, hill=1.11)
    md = m.descriptor()
    assert md.hill_mask == (1 << 2) | (1 << 3)
    assert md.hill_starmass == 1.11
    m, _ = model_51peg(peg_arr, k=3, par=0)
    assert m.descriptor().hill_mask == 0


def test_simulation_attaches_hill_per_block(peg_arr):
    from astroemperor_gb300.simulation import Simulation
    sim = Simulation()
    sim.load_arrays([peg_arr], ['51peg.vels'])
    sim.switch_dynamics = True
    sim.starmass = 1.11
    for _ in range(3):
        sim.add_keplerian()
    hills = [[ap.prargs for ap in b.additional_parameters if ap.name == 'Hill'] for b in sim.blocks__]
    # block_repo.py:611-626 runs for each block with kplan > 1
    assert hills == [[], [[2, 1.11]], [[3, 1.11]]]


def test_kat_hill_cases_reject_some_draws(kat):
    for name in ('51peg_k2_hill', '51peg_k3_hill_p0'):
        lp = kat[f'{name}__logprior']
        assert np.isfinite(lp).sum() >= 5, name
        assert (~np.isfinite(lp)).sum() >= 5, name
