"""The astrometric oracle against the reference's own code: loglike_AM of the
HIP 21850 model (tests/golden/am_kat.npz, written by tests/golden/make_golden.py
by executing the text ReddModel._write_model_AM writes, with
support/astrometry/constants.scr, on the data arrays of this package's
loader).  The reference converts mas to degrees in long double; the oracle
stays in FP64 (relative 1e-11).  And the notebook's recorded fit decomposes
as the notebook printed it."""
import os

import numpy as np
import pytest

from oracle import am as oam
from oracle.rv import OracleRV
from tests.golden.cases import HIP_MAP, model_hip21850

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


@pytest.fixture(scope='module')
def hip():
    fix = np.load(os.path.join(GOLDEN, 'hip21850.npz'))
    model, data, am = model_hip21850(fix)
    return model, data, am, OracleRV(model.spec(), dict(data.as_dict(), am=am.as_dict()))


@pytest.mark.parametrize('planets', [1, 2])
def test_loglike_am_equals_the_reference_functions(planets):
    fix = np.load(os.path.join(GOLDEN, 'hip21850.npz'))
    model, data, am = model_hip21850(fix, planets)
    pre = '' if planets == 1 else 'k2__'
    k = {key[len(pre):]: v for key, v in np.load(os.path.join(GOLDEN, 'am_kat.npz')).items()
         if key.startswith(pre) and (pre or not key.startswith('k2__'))}
    o = OracleRV(model.spec(), dict(data.as_dict(), am=am.as_dict()))
    got = []
    for t in k['theta']:
        f = o.full_theta(t)
        planets_th = [f[b.slice] for b in model.blocks if b.type_ == 'Keplerian']
        off = [f[b.slice] for b in model.blocks if b.type_ == 'AstrometryOffset'][0]
        jit = [f[b.slice] for b in model.blocks if b.type_ == 'AstrometryJitter'][0]
        got.append(oam.loglike_am(am.as_dict(), planets_th, off, jit))
    ref = k['loglike_am_ref']
    fin = np.isfinite(ref)
    assert fin.sum() >= 30
    np.testing.assert_allclose(np.array(got)[fin], ref[fin], rtol=1e-11)


def test_recorded_fit_decomposes_as_recorded(hip):
    """tests/03_hip21850_test.ipynb: maximum posterior -700.428, likelihood
    at it -642.157, so the prior there is -58.271; at the printed (rounded)
    fit the oracle's prior agrees to the rounding and the likelihood lies
    within the rounding of the maximum."""
    model, data, am, o = hip
    x = np.array(HIP_MAP)
    assert o.my_prior(x) == pytest.approx(-58.271, abs=0.02)
    assert o.my_likelihood(x) == pytest.approx(-642.157, abs=0.5)
    assert data.ndata == 97 and model.ndim__ == 23
    assert data.common_t == pytest.approx(2451118.09737, abs=1e-5)


def test_astrometry_data_shapes(hip):
    model, data, am, o = hip
    assert am.n_hipp == 108 and am.n_gost == 40
    assert int(am.masks['GDR2'].sum()) == 17 and int(am.masks['GDR3'].sum()) == 32
    assert am.gsv['GDR2'].shape == (5, 17) and am.gsv['GDR3'].shape == (5, 32)
    np.testing.assert_allclose(am.astro_gost[1, :2], 0.0)


def test_fp64_rounding_of_the_reference_formulas(hip):
    """The reference's formulas in FP64 against the same formulas with the
    barycentre and scan-epoch propagation in long double (the fixture's
    logl_ld, recomputed here): they differ by the FP64 rounding of ~60-degree
    positions, at most a few 1e-9 of the log-likelihood on these points
    (measured 4.2e-9), which is the scale the device's astrometric term is
    measured against."""
    model, data, am, o = hip
    k = np.load(os.path.join(GOLDEN, 'am_kat.npz'))
    fin = np.isfinite(k['logprior'])
    o.am_dtype = np.longdouble
    try:
        ld = np.array([o.my_likelihood(t) for t in k['theta'][fin]])
    finally:
        o.am_dtype = np.float64
    if np.finfo(np.longdouble).eps < 1e-18:
        np.testing.assert_allclose(ld, k['logl_ld'][fin], rtol=1e-14)
    rel = np.abs(k['logl'][fin] - k['logl_ld'][fin]) / np.abs(k['logl_ld'][fin])
    print(f'FP64 reference formulas against long double: median {np.median(rel):.2e} max {rel.max():.2e}')
    assert rel.max() <= 1e-8
