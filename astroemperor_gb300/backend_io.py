"""Saving and reading a finished parallel-tempering run in the layout of the
reference's post-run backend file.

EMPEROR's ``_save_backend`` (``src/astroemperor/emp.py:722-770``) writes, after
a reddemcee run, one group for the whole sampler (attribute ``iteration``;
datasets ``tsw_history`` and ``smd_history``) and one group per temperature
(datasets ``chain`` [iterations, nwalkers, ndim], ``log_like`` and
``log_prob`` [iterations, nwalkers], ``beta_history`` [iterations],
``accepted`` [nwalkers]; attribute ``iteration``).  ``save_run`` writes that
layout to HDF5 when h5py is importable and the path ends in ``.h5``, and
otherwise to a ``.npz`` archive whose keys are ``<group>/<dataset>``;
``load_run`` reads either back into a dict of the same keys.  Group names:
``mcmc`` for the sampler, ``mcmc_t<t>`` for temperature t.
"""
from __future__ import annotations

import json
import os

import numpy as np


def run_arrays(sampler, discard=0, thin=1) -> dict:
    """``<group>/<dataset>`` -> array for a finished ``PTSampler``."""
    out = {}
    n = sampler.iteration
    out['mcmc/@iteration'] = np.int64(n)
    if sampler.tsw_history_bool:
        out['mcmc/tsw_history'] = sampler.get_tsw(discard=discard, thin=thin)
    if sampler.smd_history_bool:
        out['mcmc/smd_history'] = sampler.get_smd(discard=discard, thin=thin)
    chain = sampler.get_chain(discard=discard, thin=thin)
    ll = sampler.get_log_like(discard=discard, thin=thin)
    lp = sampler.get_log_prob(discard=discard, thin=thin)
    bh = sampler.get_betas(discard=discard, thin=thin)
    acc = sampler.accepted
    for t in range(sampler.ntemps):
        g = f'mcmc_t{t}'
        out[f'{g}/@iteration'] = np.int64(n)
        out[f'{g}/chain'] = chain[t]
        out[f'{g}/log_like'] = ll[t]
        out[f'{g}/log_prob'] = lp[t]
        out[f'{g}/beta_history'] = bh[:, t]
        out[f'{g}/accepted'] = acc[t]
    return out


def _have_h5py():
    try:
        import h5py  # noqa: F401
        return True
    except ImportError:
        return False


def save_run(sampler, path, discard=0, thin=1) -> str:
    """Write the run; returns the path written (``.npz`` when HDF5 is unavailable)."""
    arrays = run_arrays(sampler, discard=discard, thin=thin)
    meta = {'ntemps': sampler.ntemps, 'nwalkers': sampler.nwalkers, 'ndim': sampler.ndim,
            'tsw_history': bool(sampler.tsw_history_bool), 'smd_history': bool(sampler.smd_history_bool)}
    if path.endswith('.h5') and _have_h5py():
        import h5py
        with h5py.File(path, 'w') as f:
            f.attrs['meta'] = json.dumps(meta)
            for key, val in arrays.items():
                grp, name = key.split('/')
                g = f.require_group(grp)
                if name.startswith('@'):
                    g.attrs[name[1:]] = int(val)
                else:
                    g.create_dataset(name, data=val)
        return path
    if path.endswith('.h5'):
        path = path[:-3] + '.npz'
    np.savez(path, __meta__=json.dumps(meta), **arrays)
    return path


def load_run(path) -> dict:
    """``<group>/<dataset>`` -> array (attributes as ``<group>/@<name>``), plus ``meta``."""
    if path.endswith('.h5'):
        import h5py
        out = {}
        with h5py.File(path, 'r') as f:
            out['meta'] = json.loads(f.attrs['meta'])
            for gname, g in f.items():
                for k, v in g.attrs.items():
                    out[f'{gname}/@{k}'] = np.int64(v)
                for dname, d in g.items():
                    out[f'{gname}/{dname}'] = d[()]
        return out
    with np.load(path, allow_pickle=False) as z:
        out = {k: z[k] for k in z.files if k != '__meta__'}
        out['meta'] = json.loads(str(z['__meta__']))
    return out
