"""Post-run backend file: the layout of the reference's ``_save_backend``
(emp.py:722-770), written and read back."""
import numpy as np
import pytest

from astroemperor_gb300.backend_io import load_run, run_arrays, save_run


class FakeRun:
    """The accessors of a finished PTSampler, on host arrays."""

    def __init__(self, T=3, W=4, D=2, S=5, seed=0):
        rng = np.random.default_rng(seed)
        self.ntemps, self.nwalkers, self.ndim, self.iteration = T, W, D, S
        self.tsw_history_bool = self.smd_history_bool = True
        self._chain = rng.normal(size=(T, S, W, D))
        self._ll = rng.normal(size=(T, S, W))
        self._lp = rng.normal(size=(T, S, W))
        self._b = np.tile(0.5 ** np.arange(T), (S, 1))
        self._tsw = rng.uniform(size=(S, T - 1))
        self._smd = rng.uniform(size=(S, T - 1))
        self.accepted = rng.integers(0, 5, size=(T, W))

    def _h(self, x, discard, thin, axis):
        sl = [slice(None)] * x.ndim
        sl[axis] = slice(discard, None, thin)
        return x[tuple(sl)]

    def get_chain(self, discard=0, thin=1):
        return self._h(self._chain, discard, thin, 1)

    def get_log_like(self, discard=0, thin=1):
        return self._h(self._ll, discard, thin, 1)

    def get_log_prob(self, discard=0, thin=1):
        return self._h(self._lp, discard, thin, 1)

    def get_betas(self, discard=0, thin=1):
        return self._h(self._b, discard, thin, 0)

    def get_tsw(self, discard=0, thin=1):
        return self._h(self._tsw, discard, thin, 0)

    def get_smd(self, discard=0, thin=1):
        return self._h(self._smd, discard, thin, 0)


def test_layout_matches_the_reference_save():
    run = FakeRun()
    a = run_arrays(run)
    assert int(a['mcmc/@iteration']) == 5
    assert a['mcmc/tsw_history'].shape == (5, 2)
    for t in range(3):
        assert a[f'mcmc_t{t}/chain'].shape == (5, 4, 2)
        assert a[f'mcmc_t{t}/log_like'].shape == (5, 4)
        assert a[f'mcmc_t{t}/beta_history'].shape == (5,)
        assert a[f'mcmc_t{t}/accepted'].shape == (4,)
        np.testing.assert_array_equal(a[f'mcmc_t{t}/chain'], run._chain[t])


def test_round_trip(tmp_path):
    run = FakeRun()
    path = save_run(run, str(tmp_path / 'star_run.h5'))
    back = load_run(path)
    assert back['meta']['ntemps'] == 3
    for k, v in run_arrays(run).items():
        np.testing.assert_array_equal(back[k], v)
    # discard / thin as the accessors take them
    path = save_run(run, str(tmp_path / 'thin.npz'), discard=1, thin=2)
    back = load_run(path)
    np.testing.assert_array_equal(back['mcmc_t1/chain'], run._chain[1, 1::2])
