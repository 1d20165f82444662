"""The oracle against its committed known-answer vectors (tests/golden).

The vectors were produced by tests/golden/make_golden.py; this keeps the
oracle stable across machines and edits.  The same cases drive the GPU
parity tests.
"""
import json

import numpy as np
import pytest

from oracle.rv import OracleRV
from tests.golden.cases import kat_cases


@pytest.fixture(scope='module')
def cases(peg_arr):
    return kat_cases(peg_arr)


def test_cases_regenerate_identically(cases, kat):
    specs = json.loads(str(kat['specs_json']))
    assert set(specs) == set(cases)
    for name, (spec, data, th) in cases.items():
        assert np.array_equal(kat[f'{name}__theta'], th), name
        assert json.loads(json.dumps(spec)) == specs[name], name


def test_oracle_matches_kat(cases, kat):
    for name, (spec, data, th) in cases.items():
        o = OracleRV(spec, data)
        lp = np.array([o.my_prior(t) for t in th])
        ll = np.array([o.my_likelihood(t) if np.isfinite(p) else -np.inf for t, p in zip(th, lp)])
        np.testing.assert_allclose(lp, kat[f'{name}__logprior'], rtol=1e-13, atol=1e-13, err_msg=name)
        np.testing.assert_allclose(ll, kat[f'{name}__logl'], rtol=1e-12, atol=1e-9, err_msg=name)
        # every case has finite and -inf priors
        assert np.isfinite(lp).sum() >= 8, name
        assert (~np.isfinite(lp)).sum() >= 4, name


def test_moav_quirk_is_a_noop(cases):
    spec, data, th = cases['c2_ma1_quirk']
    o = OracleRV(spec, data)
    spec2 = json.loads(json.dumps(spec))
    spec2['blocks'] = [b for b in spec2['blocks'] if b['type'] != 'MOAV']
    o2 = OracleRV(spec2, data)
    ndim_ma = sum(len(b['params']) for b in spec['blocks'] if b['type'] == 'MOAV')
    good = [t for t in th if np.isfinite(o.my_prior(t))]
    assert len(good) >= 4
    for t in good:
        assert o.my_likelihood(t) == o2.my_likelihood(t[:len(t) - ndim_ma])


def test_moav_documented_changes_loglike(cases):
    spec, data, th = cases['c2_ma1']
    spec_q = dict(spec, moav_reference_quirk=True)
    a, b = OracleRV(spec, data), OracleRV(spec_q, data)
    t = th[-5]
    assert a.my_likelihood(t) != b.my_likelihood(t)
