"""Oracle PT engine and its Philox stream (CPU)."""
import numpy as np
import pytest

from oracle import philox as ph
from oracle.pt import OraclePT


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    kats = [
        ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
        ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
        ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
         (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
    ]
    for ctr, key, want in kats:
        got = ph.philox4x32_10(*ctr, *key)
        assert tuple(int(g) for g in got) == want


def test_uniforms_in_open_interval():
    a = np.array([0, 0xffffffff], dtype=np.uint32)
    u = ph.u53(a, a)
    assert u[0] == 0.0 and u[1] < 1.0
    assert np.all((ph.u32u(a) > 0) & (ph.u32u(a) < 1))
    assert list(ph.mulhi(np.array([0, 0xffffffff], dtype=np.uint32), 128)) == [0, 127]


def gauss_logpost(mu, sig, lo=-50, hi=50):
    def f(theta):
        theta = np.atleast_2d(theta)
        inb = np.all((theta >= lo) & (theta <= hi), axis=1)
        lp = np.where(inb, 0.0, -np.inf)
        ll = np.where(inb, -0.5 * np.sum(((theta - mu) / sig) ** 2, axis=1), -np.inf)
        return ll, lp
    return f


@pytest.mark.parametrize('rng', ['philox', 'numpy'])
def test_tempered_gaussian_moments(rng):
    """With logP = beta logL over a flat box, temperature t samples
    N(mu, sig^2 / beta_t): check mean and variance per temperature."""
    D, T, W = 3, 4, 64
    mu, sig = np.array([1.0, -2.0, 0.5]), np.array([0.5, 1.0, 2.0])
    betas = np.array([1.0, 0.5, 0.25, 0.1])
    pt = OraclePT(gauss_logpost(mu, sig), T, W, D, betas, adapt=False, rng=rng, seed=11)
    r = np.random.default_rng(5)
    pt.set_positions(mu + r.normal(size=(T, W, D)) * sig)
    pt.run(1500)
    ch = np.array(pt.chain[300:])                     # [S, T, W, D]
    for t in range(T):
        x = ch[:, t].reshape(-1, D)
        sd = sig / np.sqrt(betas[t])
        assert np.all(np.abs(x.mean(0) - mu) < 0.12 * sd), (t, x.mean(0))
        assert np.all(np.abs(x.std(0) / sd - 1) < 0.12), (t, x.std(0) / sd)
    acc = pt.accepted.sum() / (T * W * 1500)
    assert 0.2 < acc < 0.9
    assert np.all(np.array(pt.tsw_hist).mean(0) > 0.1)


def test_ladder_adaptation_moves_interior_only():
    D, T, W = 2, 5, 32
    betas = np.array([1.0, 0.6, 0.3, 0.1, 0.01])
    pt = OraclePT(gauss_logpost(np.zeros(D), np.ones(D)), T, W, D, betas, adapt=True,
                  adapt_tau=100, adapt_nu=1, rng='philox', seed=3)
    pt.set_positions(np.random.default_rng(0).normal(size=(T, W, D)))
    pt.run(200)
    assert pt.betas[0] == 1.0 and pt.betas[-1] == 0.01
    assert np.all(np.diff(pt.betas) < 0)
    assert not np.allclose(pt.betas, betas)
