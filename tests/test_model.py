"""Model layer: default priors, theta layout and the compiled descriptor."""
import numpy as np
import pytest

from astroemperor_gb300 import _native as N
from astroemperor_gb300.model import MOAVBlock, ReddModel, SmartSetter, full_theta
from astroemperor_gb300 import synth
from oracle.rv import OracleRV
from tests.golden.cases import PEG_MAP_P1, model_51peg


def test_smartsetter_defaults_51peg(peg_arr):
    m, d = model_51peg(peg_arr, k=1, par=1, conditions=False)
    kb, ob, jb = m.blocks
    span = d.BJD.max() - d.BJD.min()
    assert kb[0].limits == [1.5, pytest.approx(span)]
    assert kb[1].limits[1] == pytest.approx(2 * np.std(d.RV))
    assert kb[2].limits == [0, pytest.approx(2 * np.pi)]
    assert kb[3].limits == [-1, 1] and kb[4].limits == [-1, 1]
    assert [p.is_hou for p in kb] == [False, False, False, True, True]
    assert ob[0].limits == [pytest.approx(-75.852, abs=5e-4), pytest.approx(75.852, abs=5e-4)]
    assert jb[0].prior == 'Normal' and jb[0].prargs == [5, 5]
    assert jb[0].limits[0] == 1e-5
    assert [p.name for p in kb.additional_parameters] == ['Eccentricity 1', 'Longitude 1']


def test_parameter_names_match_reference_conditions(peg_arr):
    m, d = model_51peg(peg_arr, k=1, par=1)
    names = [p.name for b in m.blocks for p in b]
    assert names == ['Period 1', 'Amplitude 1', 'Phase 1', 'Ecc_sin 1', 'Ecc_cos 1', 'Offset 1', 'Jitter 1']
    mb = MOAVBlock(2, {'order': 2, 'global': False})
    assert [p.name for p in mb][:4] == ['MACoefficient 1 Order 1', 'MATimescale 1 Order 1',
                                        'MACoefficient 1 Order 2', 'MATimescale 1 Order 2']


def test_descriptor_layout(peg_arr):
    m, d = model_51peg(peg_arr, k=1, par=1, fixed_ecc=True, acc=2)
    md = m.descriptor()
    assert md.n_full == 5 + 2 + 1 + 1 and md.n_free == 7
    assert md.n_planets == 1 and md.kep_param[0] == 1 and md.kep_slot[0] == 0
    assert list(md.full_src)[:9] == [0, 1, 2, -1, -1, 3, 4, 5, 6]
    assert md.acc_slot == 5 and md.acc_order == 2 and md.offset_slot == 7 and md.jitter_slot == 8
    assert [md.prior_slot[i] for i in range(7)] == [0, 1, 2, 5, 6, 7, 8]
    assert md.derived[0][0].kind == N.PRIOR_KIND['Uniform']
    assert md.derived[0][0].a0 == 0.0                       # ln(1/(1-0))
    assert md.derived[0][1].kind == N.EMP_PRIOR_NONE
    assert md.loglike_const == -0.5 * np.log(2 * np.pi) * 256
    p = md.prior[6]                                          # jitter Normal(5,5)
    assert p.kind == N.PRIOR_KIND["Normal"] and p.a0 == 5 and p.a1 == 0.2
    th = np.arange(7.0)
    ft = full_theta(m, th)[0]
    assert list(ft) == [0, 1, 2, 0, 0, 3, 4, 5, 6]


def test_prior_structs_reproduce_oracle_prior(peg_arr):
    """Evaluate the compiled priors with the device formula on the host."""
    m, d = model_51peg(peg_arr, k=1, par=0)
    md = m.descriptor()
    o = OracleRV(m.spec(), d.as_dict())
    rng = np.random.default_rng(1)
    lim = m.limits_free()
    for _ in range(50):
        th = rng.uniform(lim[:, 0], lim[:, 1])
        lp = 0.0
        for i in range(md.n_free):
            p = md.prior[i]
            x = th[i]
            if not (p.lo <= x <= p.hi):
                lp = -np.inf
                break
            if p.kind == 1:
                lp += -0.5 * ((x - p.a0) * p.a1) ** 2 - p.a2
            else:
                lp += p.a0
        assert lp == pytest.approx(o.my_prior(th), rel=1e-13, abs=1e-13)


def test_moav_must_follow_mean_model_blocks(peg_arr):
    m, d = model_51peg(peg_arr, k=1, par=1, moav={'order': 1, 'global': True})
    blocks = m.blocks
    with pytest.raises(ValueError):
        ReddModel([blocks[-1]] + blocks[:-1], d)


def test_synthetic_configs_shapes():
    for name, n, nins, kp in (('c1', 256, 1, 1), ('c2', 1024, 2, 3)):
        model, data, setup, truth = synth.build_model(name)
        assert data.ndata == n and data.nins == nins and model.kplan__ == kp
        assert len(truth) == model.ndim__
        counts = [int(np.sum(data.Flag == k + 1)) for k in range(nins)]
        assert counts == synth.CONFIGS[name]['split']
    model, data, setup, truth = synth.build_model('c2')
    assert model.ndim__ == 3 * 5 + 2 + 2 + 2 * 2      # 23: two (Phi, tau) pairs
    assert setup == [10, 256, 2000, 1]


def test_trend_blocks_descriptor_and_oracle(peg_arr):
    """sinusoid00 / magneticcycle00 compile to cosine terms; the oracle's
    model equals the templates' formulas."""
    from astroemperor_gb300 import _native as N
    from oracle.rv import OracleRV
    from tests.golden.cases import model_51peg
    m, d = model_51peg(peg_arr, k=1, par=1, sinusoid=True, cycle=True)
    md = m.descriptor()
    assert md.n_planets == 4
    assert list(md.kep_param[:4]) == [1, N.EMP_TERM_SINUSOID, N.EMP_TERM_CYCLE_1, N.EMP_TERM_CYCLE_2]
    assert list(md.kep_slot[:4]) == [0, 5, 8, 8]
    names = [p.name for p in m.free_parameters()]
    assert names[5:13] == ['Period 1', 'Amplitude 1', 'Phase 1', 'Period S1', 'Amplitude S1',
                           'Amplitude S2', 'Phase S1', 'Phase S2']
    span = d.BJD.max() - d.BJD.min()
    assert m.blocks[1][0].limits == [1.5, span]
    o = OracleRV(m.spec(), d.as_dict())
    th = np.array(PEG_MAP_P1[:5] + [700.0, 2.0, 0.5, 1100.0, 1.5, 0.7, 2.0, 4.0] + PEG_MAP_P1[5:])
    model, _ = o.my_model(th)
    m0, _ = OracleRV(model_51peg(peg_arr, k=1, par=1)[0].spec(), d.as_dict()).my_model(
        np.array(PEG_MAP_P1))
    X = d.BJD
    want = (m0 + 2.0 * np.cos(2 * np.pi / 700.0 * X + 0.5)
            + 1.5 * np.cos(np.pi / 1100.0 * X + 2.0) + 0.7 * np.cos(2 * np.pi / 1100.0 * X + 4.0))
    np.testing.assert_allclose(model, want, rtol=1e-13, atol=1e-12)


def test_trend_blocks_must_precede_moav(peg_arr):
    from astroemperor_gb300.model import MOAVBlock, ReddModel, SinusoidBlock, SmartSetter
    from tests.golden.cases import model_51peg
    m, d = model_51peg(peg_arr, k=1, par=1, moav={'order': 1, 'global': True})
    sb = SinusoidBlock(1)
    SmartSetter(d)(sb)
    with pytest.raises(ValueError, match='MOAV block must follow'):
        ReddModel(m.blocks + [sb], d)
