"""Reference-faithful CPU timing of the log-posterior (oracle; TEST / BENCH
INFRASTRUCTURE ONLY -- the CPU baseline leg of bench.py).

The reference evaluates one walker per Python call (``my_prior`` then
``my_likelihood`` -> ``my_model``, numpy over epochs) and maps the calls
over ``multiprocessing.Pool(ncores)`` (``support/pools/01.pool:10-12``,
``emp.py:503-517``).  This module does the same with the oracle's
restatement; the per-instrument moving-average block runs the reference's
literal loop (``support/models/moav00.model``), whose writes are discarded,
so the timed work equals the reference's.  A celerite GP likelihood runs the
compiled recursion of ``gp_semisep.c`` (the reference calls celerite2's
compiled core there).  The pool is started with the
``spawn`` method so that it is safe to create after CUDA is initialised.

Caveat: the Kepler equation is solved by the oracle's vectorised numpy
Halley iteration instead of the C++ ``kepler.solve`` of kepler.py 0.0.7.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import time

import numpy as np

from . import rv


def _init(spec, data):
    if any(b['type'] == 'Celerite2' for b in spec['blocks']):
        from . import gp
        gp.use_compiled(True)
    rv.install_global(spec, data)


def _eval(theta):
    return rv.global_logpost(theta)


def faithful_spec(spec):
    """The spec the reference would run: per-instrument MA is its no-op loop."""
    s = dict(spec)
    has_pi_ma = any(b['type'] == 'MOAV' and not b['global'] for b in spec['blocks'])
    if has_pi_ma:
        s['moav_reference_quirk'] = True
        s['faithful_quirk_loop'] = True
    return s


def time_pool(spec, data, thetas, ncores=None, min_seconds=10.0, max_seconds=30.0):
    """evals/s of the reference-faithful path over a Pool of ncores processes.

    Maps ``thetas`` repeatedly with Pool.map's default chunking (as emcee's
    ``pool.map`` over the walkers does) until at least ``min_seconds`` have
    passed.
    Returns (evals_per_second, n_evals, seconds, ncores).
    """
    ncores = int(ncores or os.cpu_count() or 1)
    ctx = mp.get_context('spawn')
    spec = faithful_spec(spec)
    with ctx.Pool(ncores, initializer=_init, initargs=(spec, data)) as pool:
        pool.map(_eval, list(thetas[:ncores]), chunksize=1)          # warm the workers
        n = 0
        t0 = time.perf_counter()
        while True:
            pool.map(_eval, list(thetas))
            n += len(thetas)
            el = time.perf_counter() - t0
            if el >= min_seconds or el >= max_seconds:
                break
    return n / el, n, el, ncores


class PoolTimer:
    """A reference-faithful pool kept open across timed steps."""

    def __init__(self, spec, data, ncores=None):
        self.ncores = int(ncores or os.cpu_count() or 1)
        ctx = mp.get_context('spawn')
        self.pool = ctx.Pool(self.ncores, initializer=_init, initargs=(faithful_spec(spec), data))

    def warm(self, thetas):
        self.pool.map(_eval, list(thetas[:self.ncores]), chunksize=1)

    def step(self, thetas):
        """Seconds to evaluate ``thetas`` (Pool.map's default chunking)."""
        t0 = time.perf_counter()
        self.pool.map(_eval, list(thetas))
        return time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()


def time_single(spec, data, thetas, min_seconds=2.0):
    """Single-process evals/s (no pool)."""
    o = rv.OracleRV(faithful_spec(spec), data)
    n, t0 = 0, time.perf_counter()
    while True:
        for t in thetas:
            lp = o.my_prior(t)
            if np.isfinite(lp):
                o.my_likelihood(t)
            n += 1
        el = time.perf_counter() - t0
        if el >= min_seconds:
            return n / el, n, el


def _init_many(specs, datas):
    _MANY.clear()
    _MANY.extend(rv.OracleRV(faithful_spec(sp), d) for sp, d in zip(specs, datas))


_MANY = []


def _eval_many(task):
    s, theta = task
    o = _MANY[s]
    lp = o.my_prior(theta)
    if lp == -np.inf:
        return -np.inf, lp
    return o.my_likelihood(theta), lp


def time_pool_many(specs, datas, tasks, n_epochs, ncores=None, min_seconds=10.0, max_seconds=30.0):
    """Reference-faithful CPU rate over several independent systems: each
    task (system index, theta) is one walker evaluation, as running the
    reference once per system would do.  Returns (evals*epochs per second,
    n_evals, seconds, ncores)."""
    ncores = int(ncores or os.cpu_count() or 1)
    ctx = mp.get_context('spawn')
    tasks = list(tasks)
    work = sum(int(n_epochs[s]) for s, _ in tasks)
    with ctx.Pool(ncores, initializer=_init_many, initargs=(specs, datas)) as pool:
        pool.map(_eval_many, tasks[:ncores], chunksize=1)
        n, units = 0, 0
        t0 = time.perf_counter()
        while True:
            pool.map(_eval_many, tasks)
            n += len(tasks)
            units += work
            el = time.perf_counter() - t0
            if el >= min_seconds or el >= max_seconds:
                break
    return units / el, n, el, ncores


class PoolTimerMany:
    """A reference-faithful pool over several systems kept open across steps."""

    def __init__(self, specs, datas, ncores=None):
        self.ncores = int(ncores or os.cpu_count() or 1)
        ctx = mp.get_context('spawn')
        self.pool = ctx.Pool(self.ncores, initializer=_init_many, initargs=(specs, datas))

    def step(self, tasks):
        """Seconds to evaluate (system, theta) tasks (default chunking)."""
        t0 = time.perf_counter()
        self.pool.map(_eval_many, list(tasks))
        return time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()
