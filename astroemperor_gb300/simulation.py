"""EMPEROR's user surface for the RV + parallel-tempering path.

Mirrors the parts of ``Simulation`` (``src/astroemperor/emp.py:2240-2916``)
that drive the hot path, with the same attribute names and call order::

    sim = Simulation()
    sim.load_data('51Peg')                       # {read_loc}datafiles/51Peg/RV/*.vels
    sim.set_engine('reddemcee')
    sim.engine_config['setup'] = [10, 256, 2048, 1]
    sim.keplerian_parameterisation = 1
    sim.add_condition(['Period 1', 'limits', [3, 5]])
    sim.autorun(0, 1)

Instead of writing a temporary script and running it in a child
interpreter (``emp.py:137-175, 2559-2582``), ``run`` compiles the model
(:class:`~astroemperor_gb300.model.ReddModel`) and runs the GPU
:class:`~astroemperor_gb300.engine.PTSampler` in-process.  Plotting,
logging and astrometry blocks are not part of this path.
"""
from __future__ import annotations

import itertools
import time

import numpy as np

from .data import RVData, load_target, preprocess_instruments
from .model import (AccelerationBlock, AstrometryJitterBlock, AstrometryKeplerianBlock, AstrometryOffsetBlock,
                    CeleriteBlock, JitterBlock, KeplerianBlock, MagneticCycleBlock, MOAVBlock, OffsetBlock,
                    ReddModel, SinusoidBlock, SmartSetter, full_theta)
from .stats import model_stats


class Simulation:
    def __init__(self):
        # emp.py:33-133 defaults used on this path
        self.starname = None
        self.read_loc = ''
        self.save_loc = ''
        self.blocks__ = []
        self.conds = []
        self.kplanets__ = 0
        self.nins__ = 0
        self.acceleration = 0
        self.keplerian_parameterisation = 0
        self.switch_jitter = True
        self.switch_first_run = True
        self.moav = {'order': 0, 'global': False}
        # None: as the reference computes it -- its per-instrument MA template
        # writes into a masked copy and leaves the model unchanged
        # (moav00.model:18-19), its global one is live (moav01.model).  False
        # opts in to the documented per-instrument recurrence; True forces the
        # no-op form.
        self.moav_reference_quirk = None
        self.switch_celerite = False
        self.my_kernel = {'terms': ['RealTerm'], 'params': [{'a': None, 'c': None}]}
        self.sinusoid = 0
        self.magnetic_cycle = 0
        self.eccentricity_limits = [0, 1]
        self.eccentricity_prargs = [0, 0.1]
        self.jitter_limits = [0, 1]
        self.jitter_prargs = [5, 5]
        self.instrument_names_RV = None
        # joint astrometry (emp.py:2279-2281): switched on by an AM folder
        # next to the RV one; Gaia's astrometric-gap tables (DR2, EDR3) as
        # (start, end) arrays or file paths, which the reference ships in its
        # support/deadtime folder
        self.switch_AM = False
        self.switch_inclination = False
        self.gaia_deadtime = None
        self.am_data = None
        self.starmass = 1.
        self.switch_dynamics = False
        self.dynamics_already_included = False
        self.cores__ = 1
        # emp.py:104-112: point estimate and the between-run limit constraint
        self.use_fit = 'max_post'
        self.constrain = {'method': 'range', 'sigma': 3, 'types': ['Keplerian', 'Jitter'],
                          'tol': 1e-4, 'known_methods': ['sigma', 'range', 'None']}
        self.switch_evidence = True
        self.evidence = (0.0, 0.0)
        self.engine__ = None
        self.engine_config = {}
        self.run_config = {}
        self._crit_current = 'BIC'
        self._crit_tolerance = 5
        self.BIC = np.inf
        self.like_max = -np.inf
        self.post_max = -np.inf
        self.sampler = None
        self.model = None
        self.my_data = None
        self.history = []
        self.time_run = 0.0

    # ------------------------------------------------------------------ data
    def load_data(self, folder_name):
        """emp.py:2263-2312: the RV folder, and an AM folder when present
        (qol_utils.py:103-455, astrometry.load_am)."""
        import os
        self.starname = folder_name
        self.my_data = load_target(folder_name, read_loc=self.read_loc)
        self._after_data()
        am_dir = f'{self.read_loc}datafiles/{folder_name}/AM/'
        if os.path.isdir(am_dir):
            from .astrometry import load_am, read_deadtime
            if self.gaia_deadtime is None:
                raise ValueError('astrometry needs the Gaia DR2 and EDR3 astrometric-gap tables: set '
                                 'gaia_deadtime = (dr2, edr3) as (start, end) arrays or file paths')
            dead = [read_deadtime(x) if isinstance(x, str) else x for x in self.gaia_deadtime]
            self.am_data = load_am(am_dir, dead[0], dead[1], self.my_data.common_t)
            self.switch_AM = True
            self.switch_inclination = True

    def load_arrays(self, instruments, labels=None, name='custom'):
        """Same as load_data for in-memory per-instrument (BJD, RV, eRV) arrays."""
        self.starname = name
        self.my_data = preprocess_instruments(instruments, labels)
        self._after_data()

    def _after_data(self):
        self.nins__ = self.my_data.nins
        if self.instrument_names_RV is None:
            self.instrument_names_RV = list(self.my_data.labels)
        self.my_data_common_t = self.my_data.common_t
        self.SmartSetter = SmartSetter(self.my_data)

    # ---------------------------------------------------------------- engine
    def set_engine(self, eng):
        """emp.py:2315-2388; 'reddemcee' selects the GPU PT engine."""
        if eng != 'reddemcee':
            raise ValueError(f'engine {eng!r}: only reddemcee is on the GPU path')
        from . import engine as _engine
        self.engine__ = _engine
        self.engine__.__name__ = 'reddemcee'
        self.engine_config = {'setup': np.array([5, 100, 500, 2]), 'ntemps': 5, 'betas': None,
                              'moves': None, 'tsw_history': True, 'smd_history': True,
                              'adapt_tau': 1000, 'adapt_nu': 1, 'adapt_mode': 0,
                              'progress': True, 'precision': 'mixed', 'seed': None,
                              'use_graph': True}
        self.run_config = {'burnin': None, 'adaptation_batches': None, 'adaptation_nsweeps': None,
                           'thin': 1, 'discard': 0.5, 'logger_level': 'CRITICAL',
                           # 'freeze1' (the reference's choice, emp.py:692-704) or 'batches'
                           # (support/endit_freeze.scr)
                           'adaptation_driver': 'freeze1'}
        self.evidence_method = 'hybrid'                    # emp.py:127-129

    # ---------------------------------------------------------------- blocks
    def add_keplerian(self):
        """emp.py:1212-1236; Keplerian blocks go in front of the data blocks
        (astrometric Keplerians with inclination and node when astrometry is
        on, parameterisation 0)."""
        self.kplanets__ += 1
        if self.switch_inclination:
            if self.keplerian_parameterisation != 0:
                raise ValueError('astrometric Keplerians use parameterisation 0')
            kb = AstrometryKeplerianBlock(self.kplanets__)
        else:
            kb = KeplerianBlock(self.keplerian_parameterisation, self.kplanets__)
        self.SmartSetter(kb, ecc_limits=self.eccentricity_limits, ecc_prargs=self.eccentricity_prargs,
                         starmass=self.starmass, dynamics=self.switch_dynamics, kplan=self.kplanets__,
                         dynamics_already_included=self.dynamics_already_included)
        self.blocks__.insert(self.kplanets__ - 1, kb)

    def add_offset(self):
        b = OffsetBlock(self.nins__)
        self.SmartSetter(b)
        self.blocks__.append(b)

    def add_jitter(self):
        b = JitterBlock(self.nins__)
        self.SmartSetter(b, jit_prargs=self.jitter_prargs)
        self.blocks__.append(b)

    def add_moav(self):
        b = MOAVBlock(self.nins__, self.moav)
        self.SmartSetter(b)
        self.blocks__.append(b)

    def add_offset_am(self):
        """emp.py:1307-1310."""
        b = AstrometryOffsetBlock()
        self.SmartSetter(b)
        self.blocks__.append(b)

    def add_jitter_am(self):
        """emp.py:1300-1304."""
        b = AstrometryJitterBlock()
        self.SmartSetter(b)
        self.blocks__.append(b)

    def add_acceleration(self):
        b = AccelerationBlock(self.acceleration)
        self.SmartSetter(b)
        self.blocks__.append(b)

    def add_celerite(self):
        """emp.py:1283-1296: a celerite2 GP over the residuals, hyperparameters
        from ``my_kernel``."""
        b = CeleriteBlock(self.my_kernel)
        self.SmartSetter(b)
        self.blocks__.append(b)

    def add_sinusoid(self):
        b = SinusoidBlock(self.sinusoid)
        self.SmartSetter(b)
        self.blocks__.append(b)

    def add_magnetic_cycle(self):
        b = MagneticCycleBlock(self.magnetic_cycle)
        self.SmartSetter(b)
        self.blocks__.append(b)

    def _autorun_add_RV_ins(self):
        """emp.py:2628-2650 (the blocks of this path, in the same order; the
        astrometry-correction block is not on it)."""
        if self.acceleration:
            self.add_acceleration()
        self.add_offset()
        if self.switch_jitter:
            self.add_jitter()
        if self.moav['order']:
            self.add_moav()
        if self.switch_celerite:
            self.add_celerite()
        if self.sinusoid:
            self.add_sinusoid()
        if self.magnetic_cycle:
            self.add_magnetic_cycle()

    # ------------------------------------------------------------ conditions
    def add_condition(self, cond):
        self.conds.append(cond)

    def apply_conditions(self):
        """emp.py:2790-2806: set attribute c[1] of parameter named c[0]."""
        applied = []
        for b in self.blocks__:
            for p in itertools.chain(b, getattr(b, 'additional_parameters', [])):
                for c in self.conds:
                    if p.name == c[0]:
                        setattr(p, c[1], c[2])
                        if c not in applied:
                            applied.append(c)
        for ap in applied:
            if ap in self.conds:
                self.conds.remove(ap)

    def moav_quirk(self) -> bool:
        """Whether the per-instrument MA runs as the reference's no-op."""
        if self.moav_reference_quirk is None:
            return not self.moav['global']
        return bool(self.moav_reference_quirk)

    def update_model(self):
        self.model = ReddModel(self.blocks__, self.my_data, moav_reference_quirk=self.moav_quirk(),
                               am_data=self.am_data if self.switch_AM else None)

    # ------------------------------------------------------------ init walkers
    def set_init(self, rng=np.random):
        """emp.py:617-648: stratified uniform draws in init_pos or limits."""
        ntemps, nwalkers = int(self.engine_config['setup'][0]), int(self.engine_config['setup'][1])
        free = self.model.free_parameters()
        pos = np.zeros((ntemps, nwalkers, len(free)))
        for t in range(ntemps):
            for j, p in enumerate(free):
                r = 0.707 if p.is_hou else 1
                b = p.limits[0] if p.init_pos[0] is None else np.round(p.init_pos[0], 8)
                a = p.limits[1] if p.init_pos[1] is None else np.round(p.init_pos[1], 8)
                m = (a + b) / 2
                r = (a - b) / 2 * r
                dist = np.sort(rng.uniform(0, 1, nwalkers))
                pos[t][:, j] = r * (2 * dist - 1) + m
                rng.shuffle(pos[t, :, j])
        return pos

    def test_init(self, ctx, max_repeats=100):
        """emp.py:651-681: redraw walkers whose prior is -inf (prior on the GPU)."""
        import torch
        p0 = self.set_init()
        T, W, D = p0.shape
        for _ in range(max_repeats):
            th = torch.from_numpy(p0.reshape(-1, D)).to(ctx.device)
            _, lp = ctx.logpost(th, precision=0)
            bad = ~np.isfinite(lp.cpu().numpy()).reshape(T, W)
            if not bad.any():
                return p0
            fresh = self.set_init()
            p0[bad] = fresh[bad]
        print('COULDNT FIND VALID INITIAL POSITION')
        return p0

    # ------------------------------------------------------------------- run
    def _discard(self):
        ntemps, nwalkers, nsweeps, nsteps = map(int, self.engine_config['setup'])
        niter = int(nsteps * nsweeps)
        bi = self.run_config['burnin']
        if isinstance(bi, float):
            return int(bi * niter)
        if isinstance(bi, int):
            return bi
        return 0

    def run(self):
        """emp.py:2463-2478: prepare, run the engine, keep the sampler."""
        t0 = time.time()
        self.apply_conditions()
        self.update_model()
        ntemps, nwalkers, nsweeps, nsteps = map(int, self.engine_config['setup'])
        ec = self.engine_config
        betas = ec['betas']
        if betas is not None and len(betas) != ntemps:
            raise ValueError(f'betas should have {ntemps} items')
        self.sampler = self.engine__.PTSampler(
            nwalkers, self.model.ndim__, self.model, ntemps=ntemps, betas=betas,
            tsw_history=ec['tsw_history'], smd_history=ec['smd_history'],
            adapt_tau=ec['adapt_tau'], adapt_nu=ec['adapt_nu'], adapt_mode=ec['adapt_mode'],
            precision=ec.get('precision', 'mixed'), seed=ec.get('seed'),
            use_graph=ec.get('use_graph', True))
        lim = self.model.limits_free()
        self.sampler.D_ = np.diff(lim).flatten()          # emp.py:595-602
        p1 = self.test_init(self.sampler.ctx)
        self.reddemcee_discard = self._discard()
        self.reddemcee_thin = int(self.run_config['thin'])
        ab, an = self.run_config['adaptation_batches'], self.run_config['adaptation_nsweeps']
        if ab and an and self.run_config.get('adaptation_driver') == 'batches':
            # endit_freeze.scr: adaptation batches until the autocorrelation
            # times settle, freeze, production
            self.sampler.run_adaptation_batches(p1, ab, an, nsweeps, nsteps=nsteps)
        elif ab and an:
            # endit_freeze1.scr: adaptation burn-in, freeze, production
            n1 = self.reddemcee_discard
            state = self.sampler.run_mcmc(p1, nsweeps=n1, nsteps=nsteps)
            self.sampler.select_adjustment('00')
            self.sampler.run_mcmc(state, nsweeps=nsweeps - n1, nsteps=nsteps)
        else:
            self.sampler.run_mcmc(p1, nsweeps=nsweeps, nsteps=nsteps)
        self.time_run = time.time() - t0

    def postprocess(self):
        """emp.py:1324-1340 without the plots and logs: samples, evidence, the
        point estimates of ``_get_fit_reddemcee`` (emp.py:1467-1496), the
        statistics of ``_calculate_statistics`` (emp.py:1546-1557,
        1187-1210) and the per-parameter values of ``_set_p_values``
        (emp.py:1560-1566, 1721-1767)."""
        from .stats import hdi_of_chain
        d = dict(discard=self.reddemcee_discard, thin=self.reddemcee_thin, flat=True)
        self.chain = self.sampler.get_chain(**d)
        self.likes = self.sampler.get_log_like(**d)
        self.posts = self.sampler.get_log_prob(**d)
        if self.switch_evidence:
            # emp.py:1431-1446: the configured estimator, then TI, then TI
            # without the PCHIP interpolation
            method = getattr(self, 'evidence_method', 'hybrid')
            try:
                z = getattr(self.sampler, f'get_evidence_{method}')(discard=self.reddemcee_discard)[:2]
                if z[0] == -np.inf:
                    z = self.sampler.get_evidence_ti(discard=self.reddemcee_discard)[:2]
                if z[0] == -np.inf:
                    z = self.sampler.get_evidence_ti(discard=self.reddemcee_discard, pchip=False)[:2]
            except Exception:
                z = self.sampler.get_evidence_ti(discard=self.reddemcee_discard, pchip=False)[:2]
            self.evidence = (z[0], z[1])
        ch0 = self.chain[0]
        self.best_loc_post = int(np.argmax(self.posts[0]))
        self.best_loc_like = int(np.argmax(self.likes[0]))
        # the "maximum likelihood" the reference reports, and the one its BIC
        # uses, is the likelihood of the maximum-posterior sample
        self.post_max = float(self.posts[0][self.best_loc_post])
        self.like_max = float(self.likes[0][self.best_loc_post])
        self.prior_max_post = self.post_max - self.like_max
        self.sigmas = np.std(ch0, axis=0)
        self.fit_max = ch0[self.best_loc_post]
        self.fit_mean = np.mean(ch0, axis=0)
        self.fit_median = np.median(ch0, axis=0)
        self.fit_low1, self.fit_high1 = hdi_of_chain(ch0, 0.36).T
        self.fit_low2, self.fit_high2 = hdi_of_chain(ch0, 0.90).T
        self.fit_low3, self.fit_high3 = hdi_of_chain(ch0, 0.95).T
        self.fit_maxlike = ch0[self.best_loc_like]
        self.fit_like = self.fit_maxlike
        self.ajuste = {'max_post': self.fit_max, 'max_like': self.fit_maxlike, 'mean': self.fit_mean,
                       'median': self.fit_median}.get(self.use_fit, self.fit_max)
        resid, err2 = self.residuals(self.ajuste)
        st = model_stats(resid, err2, self.model.ndim__, self.like_max,
                         flags=self.my_data.Flag, nins=self.nins__)
        for k, v in st.items():
            setattr(self, k, v)
        # emp.py:1202, 1548: DIC from the likelihood at the posterior mean
        self.dic_aux = float(np.var(-2 * self.likes[0]))
        self.DIC = -2 * self.log_like_at(self.fit_mean) + self.dic_aux
        self.Evidence = self.evidence[0]
        self.post_true = self.post_max - self.Evidence
        self.BayesFactor = self.like_max - self.Evidence
        self._set_p_values()
        self.history.append({'k': self.kplanets__, 'like_max': self.like_max,
                             'post_max': self.post_max, 'BIC': self.BIC, 'fit': self.fit_max,
                             'evidence': self.evidence})

    def _set_p_values(self):
        """emp.py:1560-1566, 1721-1767: value, sigma, HDI bounds and the
        1-sigma ``value_range`` of every free parameter; fixed ones get
        their value and NaN spreads."""
        j = 0
        for b in self.blocks__:
            for p in b:
                if p.fixed is not None:
                    p.sigma = np.nan
                    p.value_max = p.value_mean = p.value_median = p.value_max_lk = p.value
                    for lvl in (1, 2, 3):
                        setattr(p, f'value_low{lvl}', np.nan)
                        setattr(p, f'value_high{lvl}', np.nan)
                    p.value_range = [np.nan, np.nan]
                    continue
                p.cpointer = j
                p.value = float(self.ajuste[j])
                p.sigma = float(self.sigmas[j])
                p.value_max, p.value_mean = float(self.fit_max[j]), float(self.fit_mean[j])
                p.value_median, p.value_max_lk = float(self.fit_median[j]), float(self.fit_maxlike[j])
                for lvl in (1, 2, 3):
                    setattr(p, f'value_low{lvl}', float(getattr(self, f'fit_low{lvl}')[j]))
                    setattr(p, f'value_high{lvl}', float(getattr(self, f'fit_high{lvl}')[j]))
                a = p.value_low1 if p.value_low1 < p.value_max else p.value_max - p.sigma
                c = p.value_high1 if p.value_high1 > p.value_max else p.value_max + p.sigma
                p.value_range = [max(a, p.limits[0]), min(c, p.limits[1])]
                j += 1

    def residuals(self, theta):
        """(Y - model, err2) at theta, from the device my_model (for stats)."""
        import torch
        ctx = self.sampler.ctx
        th = torch.as_tensor(np.atleast_2d(theta), dtype=torch.float64, device=ctx.device)
        model0, err2 = ctx.model_eval(th)
        return self.my_data.RV - model0[0].cpu().numpy(), err2[0].cpu().numpy()

    def log_like_at(self, theta):
        """my_likelihood(theta) on the device (FP64)."""
        import torch
        ctx = self.sampler.ctx
        th = torch.as_tensor(np.atleast_2d(theta), dtype=torch.float64, device=ctx.device)
        ll, _ = ctx.logpost(th, precision=0)
        return float(ll[0].item())

    # ------------------------------------------------------- between runs
    def _set_init_pos(self):
        """emp.py:2671-2675: the next run starts the Keplerians inside their
        1-sigma ranges."""
        for b in self.blocks__:
            if b.type_ == 'Keplerian':
                for p in b:
                    if p.fixed is None:
                        p.init_pos = list(p.value_range)

    def _constrain_next_run(self):
        """emp.py:2707-2783 ('sigma' and 'range'; 'GM' needs the Gaussian
        mixture fits, which are not on this path): narrow the limits of the
        Keplerian and jitter parameters for the next run by conditions."""
        method = self.constrain['method']
        if method == 'None':
            return
        if method not in ('sigma', 'range'):
            raise ValueError(f'constrain method {method!r} is not on this path')
        nsig = self.constrain['sigma']
        for b in self.blocks__:
            if b.type_ not in self.constrain['types']:
                continue
            for p in b:
                if p.fixed is not None:
                    continue
                if method == 'sigma':
                    limf, limc = p.value - nsig * p.sigma, p.value + nsig * p.sigma
                else:
                    limf, limc = getattr(p, f'value_low{nsig}'), getattr(p, f'value_high{nsig}')
                limc = min(limc, p.limits[1])
                if limf < p.limits[0] or b.type_ == 'Jitter':
                    limf = p.limits[0]
                if (limc - limf) / abs(p.value) >= self.constrain['tol']:
                    self.add_condition([p.name, 'limits', [limf, limc]])

    def _check_continue_run(self, old_crit):
        """emp.py:2654-2668: False while the criterion improved by more than
        the tolerance and runs remain."""
        new = getattr(self, self._crit_current)
        if not (old_crit - new > self._crit_tolerance):
            return False
        return self.k_start <= self.k_end

    def autorun(self, k_start=0, k_end=10):
        """emp.py:2414-2456: runs of k_start..k_end Keplerians while the BIC
        improves by more than ``_crit_tolerance`` (emp.py:1145-1156); between
        runs the Keplerians start inside the last run's ranges and the
        Keplerian and jitter limits are narrowed (``constrain``)."""
        assert k_start <= k_end, f'Invalid keplerian starting point: ({k_start}, {k_end})'
        self.k_start, self.k_end = k_start, k_end
        while self.k_start <= self.k_end:
            if self.switch_first_run:
                # emp.py:2614-2625
                self._autorun_add_RV_ins()
                for _ in range(self.k_start):
                    self.add_keplerian()
                if self.switch_AM:
                    self.add_offset_am()
                    self.add_jitter_am()
                self.switch_first_run = False
            old = getattr(self, self._crit_current)
            self.run()
            self.postprocess()
            self.k_start += 1
            if not self._check_continue_run(old):
                break
            self._set_init_pos()
            self._constrain_next_run()
            self.add_keplerian()
