"""Celerite GP likelihood on the CPU: the oracle's semiseparable recursion
against the dense definition, the model layer's GP descriptor, and the
Simulation block order of the reference's GP runs.

Tolerance: recursion vs dense Cholesky, |dlogL| / |logL| <= 1e-10.
"""
import numpy as np
import pytest

from astroemperor_gb300 import _native as N
from astroemperor_gb300.model import CeleriteBlock, MOAVBlock, ReddModel
from oracle import gp
from oracle.rv import OracleRV
from tests.golden.cases import GP_KERNELS, gp_case_models, model_51peg, peg_data

RTOL = 1e-10


def _series(rng, n):
    t = np.sort(rng.uniform(0, 300, n))
    t[5] = t[4]                                    # a repeated epoch
    return t, rng.normal(0, 3, n), rng.uniform(0.5, 4, n)


TERM_CASES = [
    (gp.GP_REAL, [2.0, 0.3]),
    (gp.GP_MATERN32, [1.5, 4.0]),
    (gp.GP_ROTATION, [2.0, 12.0, 0.8, 1.5, 0.4]),
    (gp.GP_GROT, [9.0, 20.0, 3.0, 1.0]),
    (gp.GP_GROT, [9.0, 0.5, 3.0, 1.0]),            # Q < 1/2: the real-component regime
    (gp.GP_SHO, [4.0, 0.9, 3.0]),                  # S0, w0, Q
    (gp.GP_SHO, [4.0, 0.9, 0.2]),                  # Q < 1/2
    (gp.GP_SHO + 7, [2.0, 7.0, 15.0]),             # sigma, rho, tau
    (gp.GP_SHO + 3, [2.0, 7.0, 0.3]),              # sigma, rho, Q
]


@pytest.mark.parametrize('kind,p', TERM_CASES)
def test_semiseparable_recursion_equals_dense(kind, p):
    rng = np.random.default_rng(kind * 31 + len(p))
    t, r, diag = _series(rng, 120)
    co = gp.coefficients([(kind, p)])
    a = gp.semisep_loglike(t, r, diag, co)
    b = gp.dense_loglike(t, r, diag, co)
    assert np.isfinite(a)
    assert abs(a - b) <= RTOL * abs(b), (a, b)


def test_sum_of_terms_equals_dense():
    rng = np.random.default_rng(5)
    t, r, diag = _series(rng, 200)
    terms = [(gp.GP_REAL, [1.0, 0.05]), (gp.GP_SHO + 7, [2.0, 7.0, 15.0]), (gp.GP_GROT, [9.0, 20.0, 3.0, 1.0])]
    co = gp.coefficients(terms)
    assert len(co[0]) == 1 and len(co[2]) == 3
    a = gp.semisep_loglike(t, r, diag, co)
    b = gp.dense_loglike(t, r, diag, co)
    assert abs(a - b) <= RTOL * abs(b)


def test_zero_amplitude_terms_give_the_gaussian_likelihood():
    """A state dimension whose U is zero adds nothing to D_n or z_n, so the
    recursion of a system without GP terms (all dimensions padding, as a
    batch handle runs it beside GP systems) is the independent Gaussian
    log-likelihood -0.5 sum(r^2 / err2 + log err2) - 0.5 N log 2 pi."""
    rng = np.random.default_rng(11)
    t, r, diag = _series(rng, 150)
    gauss = -0.5 * np.sum(r * r / diag + np.log(diag)) - 0.5 * len(t) * np.log(2 * np.pi)
    for terms in ([(gp.GP_REAL, [0.0, 0.3])], [(gp.GP_SHO, [0.0, 0.9, 3.0])],
                  [(gp.GP_ROTATION, [0.0, 12.0, 0.8, 1.5, 0.4])]):
        co = gp.coefficients(terms)
        assert gp.semisep_loglike(t, r, diag, co) == pytest.approx(gauss, rel=1e-14)


def test_sho_parameterisations_agree():
    # (sigma, rho, tau) and the equivalent (S0, w0, Q) give one kernel
    sigma, rho, tau = 2.0, 7.0, 15.0
    w0 = 2 * np.pi / rho
    Q = 0.5 * w0 * tau
    S0 = sigma ** 2 / (w0 * Q)
    tau_grid = np.linspace(0, 50, 11)
    k1 = gp.kernel_value(gp.coefficients([(gp.GP_SHO + 7, [sigma, rho, tau])]), tau_grid)
    k2 = gp.kernel_value(gp.coefficients([(gp.GP_SHO, [S0, w0, Q])]), tau_grid)
    np.testing.assert_allclose(k1, k2, rtol=1e-14)
    assert abs(k1[0] - sigma ** 2) < 1e-12


def test_model_descriptor_gp_fields(peg_arr):
    m, d = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['real_matern'])
    terms = m.gp_terms()
    names = [p.name for b in m.blocks for p in b]
    assert names[-4:] == ['Real Term a1', 'Real Term c1', 'Matern32 Term sigma2', 'Matern32 Term rho2']
    assert [k for k, _ in terms] == [N.EMP_GP_REAL, N.EMP_GP_MATERN32]
    md = m.descriptor()
    assert md.gp_nterms == 2
    assert list(md.gp_kind[:2]) == [N.EMP_GP_REAL, N.EMP_GP_MATERN32]
    assert list(md.gp_slot[0]) == terms[0][1] + [-1, -1, -1]
    assert list(md.gp_slot[1]) == terms[1][1] + [-1, -1, -1]
    # the fixed RealTerm c is a fixed slot, the others are free
    c_slot = terms[0][1][1]
    assert md.full_src[c_slot] == -1 and md.full_fixed[c_slot] == 0.5
    assert all(md.full_src[s] >= 0 for s in terms[1][1])
    # default limits of the reference's smart setter
    lim = m.limits_free()
    np.testing.assert_allclose(lim[-3:], [[1e-5, 5.0]] * 3)


def test_sho_kinds_and_rotation_mixing_limit(peg_arr):
    m, _ = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['sho_rho_tau_sigma'])
    (kind, slots), = m.gp_terms()
    assert kind == N.EMP_GP_SHO + 7
    names = [p.name for b in m.blocks for p in b]
    # canonical order (sigma, rho, tau) from the dictionary order (rho, tau, sigma)
    assert [names[s] for s in slots] == ['SHO Term sigma', 'SHO Term rho', 'SHO Term tau']
    m, _ = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['rotation'])
    lim = m.limits_free()
    np.testing.assert_allclose(lim[-1], [1e-5, 1.0])


def test_oracle_gp_likelihood_equals_dense(peg_arr):
    cases = gp_case_models(peg_arr, n_in=4, n_near=3)
    for name, (m, d, th) in cases.items():
        o = OracleRV(m.spec(), d.as_dict())
        (terms,) = [b['gp_terms'] for b in o.blocks if b['type'] == 'Celerite2']
        n_fin = 0
        for x in th:
            if not np.isfinite(o.my_prior(x)):
                continue
            model, err2 = o.my_model(x)
            full = o.full_theta(x)
            co = gp.coefficients([(k, [full[i] for i in sl]) for k, sl in terms])
            dense = gp.dense_loglike(o.X_, o.Y_ - model, err2, co)
            assert abs(o.my_likelihood(x) - dense) <= RTOL * abs(dense), name
            n_fin += 1
        assert n_fin >= 3, name


def test_gp_with_live_moav_models_the_ma_residuals(peg_arr):
    # 02.like: gp_.mean = my_model's model, which holds the MA terms of a live
    # MOAV block (moav01.model), so the GP sees the residuals after the MA
    from oracle import gp
    for moav in ({'order': 1, 'global': True}, {'order': 2, 'global': False}):
        m, d = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['grot'], moav=moav, quirk=False)
        o = OracleRV(m.spec(), d.as_dict())
        (terms,) = [b['gp_terms'] for b in o.blocks if b['type'] == 'Celerite2']
        nma = 2 * moav['order']
        x = np.concatenate([[4.231, 55.957, 1.769, 0.087, 0.061, 3.642, 2.961],
                            [0.4, 5.0] * moav['order'], [2.5, 2.5, 2.5, 2.5]])
        assert len(x) == m.ndim__
        model, err2 = o.my_model(x)
        x0 = x.copy()
        x0[7:7 + nma:2] = 0.0                                   # MA coefficients off
        model0, _ = o.my_model(x0)
        assert np.max(np.abs(model - model0)) > 0.1
        full = o.full_theta(x)
        co = gp.coefficients([(k, [full[i] for i in sl]) for k, sl in terms])
        dense = gp.dense_loglike(o.X_, o.Y_ - model, err2, co)
        assert abs(o.my_likelihood(x) - dense) <= RTOL * abs(dense)


def test_gp_with_quirk_moav_is_the_gp_alone(peg_arr):
    # the reference's per-instrument MOAV is a no-op: with the quirk the GP
    # likelihood equals that of the same model without the MOAV block
    m0, d = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['grot'])
    mq, _ = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['grot'], moav={'order': 1, 'global': False},
                        quirk=True)
    o0 = OracleRV(m0.spec(), d.as_dict())
    oq = OracleRV(mq.spec(), d.as_dict())
    th0 = np.array([4.231, 55.957, 1.769, 0.087, 0.061, 3.642, 2.961, 2.5, 2.5, 2.5, 2.5])
    thq = np.concatenate([th0[:7], [0.1, 10.0], th0[7:]])     # MA coefficient and timescale
    assert abs(oq.my_likelihood(thq) - o0.my_likelihood(th0)) <= 1e-12 * abs(o0.my_likelihood(th0))
    md = mq.descriptor()
    assert md.gp_nterms == 1 and md.ma_order == 1 and md.ma_quirk == 1


def test_unknown_term_rejected():
    with pytest.raises(ValueError, match='not built'):
        CeleriteBlock({'terms': ['CosineTerm'], 'params': [{'sigma': None, 'period': None}]})


def test_simulation_block_order(peg_arr):
    from astroemperor_gb300.simulation import Simulation
    sim = Simulation()
    sim.load_arrays([peg_arr], ['51peg.vels'])
    sim.switch_celerite = True
    sim.my_kernel = GP_KERNELS['grot']
    sim.sinusoid = 1
    sim._autorun_add_RV_ins()
    # emp.py:2628-2650: offset, jitter, celerite, sinusoid
    assert [b.type_ for b in sim.blocks__] == ['Offset', 'Jitter', 'Celerite2', 'Sinusoid']


@pytest.mark.parametrize('kind,p', TERM_CASES[:5])
def test_compiled_recursion_equals_python(kind, p):
    rng = np.random.default_rng(kind + 100)
    t, r, diag = _series(rng, 150)
    co = gp.coefficients([(kind, p), (gp.GP_REAL, [0.7, 0.02])])
    a = gp.semisep_loglike(t, r, diag, co)
    b = gp.semisep_loglike_c(t, r, diag, co)
    assert abs(a - b) <= 1e-12 * abs(a), (a, b)
    # not positive definite -> -inf in both
    bad = [x.copy() if hasattr(x, 'copy') else list(x) for x in co]
    bad[0] = [-50.0] + list(bad[0])[1:]
    assert gp.semisep_loglike(t, r, diag, bad) == -np.inf
    assert gp.semisep_loglike_c(t, r, diag, bad) == -np.inf


def test_oracle_matches_gp_fixture(peg_arr):
    """The committed GP known-answer vectors (tests/golden/make_golden.py) keep
    the GP oracle stable across machines and edits."""
    kat = np.load('tests/golden/gp_kat.npz')
    cases = gp_case_models(peg_arr)
    for name, (m, d, th) in cases.items():
        np.testing.assert_array_equal(th, kat[f'{name}__theta'])
        o = OracleRV(m.spec(), d.as_dict())
        lp = np.array([o.my_prior(t) for t in th])
        np.testing.assert_allclose(lp, kat[f'{name}__logprior'], rtol=1e-13, atol=1e-13)
        fin = np.isfinite(lp)
        ll = np.array([o.my_likelihood(t) for t in th[fin]])
        np.testing.assert_allclose(ll, kat[f'{name}__logl'][fin], rtol=1e-12, err_msg=name)
