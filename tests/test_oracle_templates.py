"""The oracle against the reference's own code: my_model / my_likelihood /
my_prior of the known-answer cases as the reference's templates compute them
(my_prior assembled as emp.py:182-254 writes it, with the reference's own
prargs normaliser and Hill/PAE code), and its prior templates
(tests/golden/template_kat.npz, written by
tests/golden/make_golden.py from support/models/*.model,
support/likelihoods/00.like and support/priors/*.prior; the Kepler equation,
a third-party call absent here, solved by the oracle's solver in both).

Tolerances: model and err2 relative 1e-13 (the same operations; numpy's
pairwise sums and the oracle's vectorised forms differ in the last bits),
logL relative 1e-12, priors exact to 1e-13, my_prior bit for bit.
"""
import numpy as np
import pytest

from oracle.rv import OracleRV, PRIORS, check_prargs
from tests.golden.cases import kat_case_models


@pytest.fixture(scope='module')
def tkat():
    return np.load('tests/golden/template_kat.npz')


def test_oracle_model_and_likelihood_equal_reference_templates(peg_arr, tkat):
    cases = kat_case_models(peg_arr)
    names = sorted({k.split('__')[0] for k in tkat.files if k.endswith('__logl')})
    assert len(names) >= 14
    for name in names:
        m, d, th = cases[name]
        o = OracleRV(m.spec(), d.as_dict())
        pick = tkat[f'{name}__pick']
        with np.errstate(all='ignore'):
            for j, i in enumerate(pick):
                mod, err2 = o.my_model(th[i])
                ref_m, ref_e = tkat[f'{name}__model'][j], tkat[f'{name}__err2'][j]
                fin = np.isfinite(ref_m)
                np.testing.assert_allclose(mod[fin], ref_m[fin], rtol=1e-13, atol=1e-11, err_msg=name)
                np.testing.assert_allclose(err2, ref_e, rtol=1e-13, err_msg=name)
            ll = np.array([o.my_likelihood(t) for t in th])
        ref = tkat[f'{name}__logl']
        fin = np.isfinite(ref)
        assert fin.sum() >= 10, name
        np.testing.assert_allclose(ll[fin], ref[fin], rtol=1e-12, err_msg=name)


@pytest.mark.parametrize('prior', ['Uniform', 'Normal', 'Jeffreys', 'Beta'])
def test_oracle_priors_equal_reference_templates(tkat, prior):
    xin = tkat[f'prior_{prior}__in']
    want = tkat[f'prior_{prior}__value']
    fn = PRIORS[prior]
    got = []
    for row in xin:
        x, lo, hi = row[:3]
        pr = None if np.isnan(row[3]) else [row[3], row[4]]
        args = check_prargs(prior, [lo, hi], pr)
        with np.errstate(all='ignore'):
            got.append(fn(x, [lo, hi], args))
    got = np.array(got, dtype=np.float64)
    fin = np.isfinite(want)
    assert np.array_equal(np.isfinite(got), fin)
    assert fin.sum() > 20 and (~fin).sum() > 5
    np.testing.assert_allclose(got[fin], want[fin], rtol=1e-13, atol=1e-13)


def test_oracle_my_prior_equals_reference_assembly(peg_arr, tkat):
    cases = kat_case_models(peg_arr)
    names = sorted({k.split('__')[0] for k in tkat.files if k.endswith('__logprior')})
    assert '51peg_k3_hill_p0' in names and '51peg_k1_p7' in names
    for name in names:
        m, d, th = cases[name]
        o = OracleRV(m.spec(), d.as_dict())
        with np.errstate(all='ignore'):
            lp = np.array([o.my_prior(t) for t in th])
        ref = tkat[f'{name}__logprior']
        np.testing.assert_array_equal(np.isfinite(lp), np.isfinite(ref), err_msg=name)
        fin = np.isfinite(ref)
        np.testing.assert_array_equal(lp[fin], ref[fin], err_msg=name)


@pytest.mark.parametrize('quirk,case', [(None, 'c2_ma1_quirk'), (False, 'c2_ma1')])
def test_simulation_ma_default_follows_the_reference(peg_arr, tkat, quirk, case):
    """A Simulation with per-instrument MA(1) computes what the reference's
    generated my_likelihood computes (its per-instrument template is a
    no-op); ``moav_reference_quirk = False`` opts in to the documented
    recurrence, pinned to the reference's live template run per instrument."""
    from astroemperor_gb300 import synth
    from astroemperor_gb300.simulation import Simulation
    instruments, _ = synth.make_system('c2', seed=7)
    sim = Simulation()
    sim.load_arrays(instruments, ['INS1', 'INS2'])
    sim.keplerian_parameterisation = 1
    sim.moav = {'order': 1, 'global': False}
    if quirk is not None:
        sim.moav_reference_quirk = quirk
    sim._autorun_add_RV_ins()
    for _ in range(3):
        sim.add_keplerian()
    sim.apply_conditions()
    sim.update_model()
    assert sim.model.moav_reference_quirk is (quirk is None)
    m, d, th = kat_case_models(peg_arr)[case]
    assert [p.name for p in sim.model.free_parameters()] == [p.name for p in m.free_parameters()]
    o = OracleRV(sim.model.spec(), sim.my_data.as_dict())
    ref = tkat[f'{case}__logl']
    fin = np.isfinite(ref)
    with np.errstate(all='ignore'):
        ll = np.array([o.my_likelihood(t) for t in th[fin]])
    np.testing.assert_allclose(ll, ref[fin], rtol=1e-12)
