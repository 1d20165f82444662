"""Seeded synthetic RV workloads with the shapes of the benchmark configs.

There is no public data set for these workloads; each generator draws a
system from a fixed seed, with the sizes and value distributions the
configuration names, and returns per-instrument (BJD, RV, eRV) arrays that
go through the same preprocessing as EMPEROR's ``DataWrapper``.

* ``c1`` -- 51 Peg shape: 1 Keplerian, 1 instrument, N=256, T x W = 2 x 100.
* ``c2`` -- 3 Keplerians, 2 instruments (614/410 epochs), N=1024, clumpy
  nightly cadence over 3000 d, per-instrument MA(1) (Phi=0.4, tau=5 d),
  T x W = 10 x 256, 2000 sweeps.
* ``c4`` -- 5 Keplerians, 3 instruments, MA(1), N=4096.
* ``c5`` -- 7 Keplerians, 4 instruments, MA(2), N=16384 over 10000 d,
  T x W = 32 x 1024.
* ``c3`` -- a ragged batch of independent systems (``make_ragged``): epoch
  counts log-uniform in [50, 2000] over 1000-5000 d, 1-4 Keplerians with P
  log-uniform in [1, 3000] d, K log-uniform in [0.5, 100] m/s,
  e ~ Beta(0.87, 3.03), 1-3 instruments; T x W = 8 x 64, 1000 sweeps.
"""
from __future__ import annotations

import numpy as np

from .data import preprocess_instruments
from .model import (CeleriteBlock, JitterBlock, KeplerianBlock, MOAVBlock, OffsetBlock, ReddModel,
                    SmartSetter)

BJD0 = 2450000.0


def _kepler_E(M, e):
    M = np.remainder(M + np.pi, 2 * np.pi) - np.pi
    E = M + 0.85 * e * np.sign(np.sin(M))
    for _ in range(50):
        f = E - e * np.sin(E) - M
        E = E - f / (1 - e * np.cos(E))
    return E


def keplerian(t, P, K, phase, e, w):
    """K (cos(f + w) + e cos w) with M = 2 pi t / P + phase."""
    E = _kepler_E(2 * np.pi / P * t + phase, e)
    f = 2 * np.arctan(np.sqrt((1 + e) / (1 - e)) * np.tan(E / 2))
    return K * (np.cos(f + w) + e * np.cos(w))


def _clumpy_times(rng, n, span, t0=BJD0):
    """Nightly blocks (1 + Poisson(2) visits a night) with seasonal gaps."""
    times = []
    while len(times) < n:
        night = rng.uniform(0, span)
        if (night % 365.25) > 240.0:          # out of season
            continue
        k = 1 + rng.poisson(2.0)
        times.extend(night + np.sort(rng.uniform(0, 0.3, k)))
    return t0 + np.sort(np.array(times[:n]))


def _ma_noise(rng, t, sig, phis, taus):
    """White noise w plus MA terms sum_c Phi_c exp(-|dt|/tau_c) w_{i-1-c}."""
    w = rng.normal(0.0, sig)
    out = w.copy()
    for i in range(len(t)):
        for c, (phi, tau) in enumerate(zip(phis, taus)):
            if i > c:
                out[i] += phi * np.exp(-abs(t[i] - t[i - 1 - c]) / tau) * w[i - 1 - c]
    return out


CONFIGS = {
    'c1': dict(n=256, nins=1, split=[256], span=2000.0, clumpy=False,
               P=[4.2308], K=[56.0], e=[0.01], w=[1.0], offsets=[0.0], jitters=[1.5],
               ma=None, setup=[2, 100, 500, 1]),
    'c2': dict(n=1024, nins=2, split=[614, 410], span=3000.0, clumpy=True,
               P=[4.6, 61.0, 1250.0], K=[12.0, 5.0, 20.0], e=None, w=None,
               offsets=[0.0, 30.0], jitters=[1.0, 3.0], ma=dict(order=1, phi=[0.4], tau=[5.0]),
               setup=[10, 256, 2000, 1]),
    'c4': dict(n=4096, nins=3, split=[1638, 1434, 1024], span=4000.0, clumpy=True,
               P=[3.7, 12.3, 45.0, 230.0, 1500.0], K=[9.0, 6.0, 11.0, 4.0, 18.0], e=None, w=None,
               offsets=[0.0, 25.0, -15.0], jitters=[1.0, 2.0, 3.0],
               ma=dict(order=1, phi=[0.4], tau=[5.0]), setup=[8, 128, 1000, 1]),
    'c5': dict(n=16384, nins=4, split=[4916, 4096, 4096, 3276], span=10000.0, clumpy=True,
               P=[3.1, 7.9, 19.5, 48.0, 123.0, 410.0, 2100.0],
               K=[8.0, 6.0, 10.0, 4.0, 12.0, 7.0, 15.0], e=None, w=None,
               offsets=[0.0, 20.0, -10.0, 35.0], jitters=[1.0, 1.5, 2.0, 3.0],
               ma=dict(order=2, phi=[0.4, 0.2], tau=[5.0, 10.0]), setup=[32, 1024, 5000, 1]),
    # C2's planets and cadence with stellar-rotation noise instead of MA: a
    # GonzRotationTerm GP (SHO terms at the rotation period and its half)
    'gp': dict(n=1024, nins=2, split=[614, 410], span=3000.0, clumpy=True,
               P=[4.6, 61.0, 1250.0], K=[12.0, 5.0, 20.0], e=None, w=None,
               offsets=[0.0, 30.0], jitters=[1.0, 3.0], ma=None,
               gp=dict(rho=25.0, tau=50.0, A1=4.0, A2=1.5), setup=[10, 256, 2000, 1]),
}


def _sho_cov(tau, S0, w0, Q):
    """Stochastically driven damped oscillator covariance for Q > 1/2
    (Foreman-Mackey et al. 2017, eq. 20 with eta = sqrt(1 - 1/(4 Q^2)))."""
    eta = np.sqrt(1.0 - 1.0 / (4.0 * Q * Q))
    x = w0 * np.abs(tau)
    return S0 * w0 * Q * np.exp(-x / (2 * Q)) * (np.cos(eta * x) + np.sin(eta * x) / (2 * eta * Q))


def rotation_gp_noise(rng, t, gp):
    """A draw of the GonzRotationTerm GP (SHO(S0=A1, rho, tau) + SHO(S0=A2,
    rho/2, tau)) at times t, by a dense Cholesky factor."""
    tau = t[:, None] - t[None, :]
    K = np.zeros_like(tau)
    for S0, rho in ((gp['A1'], gp['rho']), (gp['A2'], 0.5 * gp['rho'])):
        w0 = 2 * np.pi / rho
        K += _sho_cov(tau, S0, w0, 0.5 * w0 * gp['tau'])
    K[np.diag_indices_from(K)] += 1e-9 * K[0, 0]
    return np.linalg.cholesky(K) @ rng.normal(size=len(t))


def make_system(name: str, seed: int = 1234):
    """(instruments, truth) of a config; truth holds the generating values."""
    cfg = CONFIGS[name]
    rng = np.random.default_rng(seed)
    n, nins = cfg['n'], cfg['nins']
    if cfg['clumpy']:
        t_all = _clumpy_times(rng, n, cfg['span'])
    else:
        t_all = BJD0 + np.sort(rng.uniform(0, cfg['span'], n))
    # instrument per epoch with the config's split, assigned by night blocks
    labels = np.repeat(np.arange(nins), cfg['split'])
    rng.shuffle(labels)
    kp = len(cfg['P'])
    e = cfg['e'] if cfg['e'] is not None else list(np.minimum(rng.beta(0.87, 3.03, kp), 0.8))
    w = cfg['w'] if cfg['w'] is not None else list(rng.uniform(0, 2 * np.pi, kp))
    phase = list(rng.uniform(0, 2 * np.pi, kp))
    tr = t_all - t_all.min()
    rv = np.zeros(n)
    for p in range(kp):
        rv += keplerian(tr, cfg['P'][p], cfg['K'][p], phase[p], e[p], w[p])
    if cfg.get('gp'):
        order = np.argsort(tr, kind='mergesort')
        g = np.empty(n)
        g[order] = rotation_gp_noise(rng, tr[order], cfg['gp'])
        rv += g
    sig = rng.uniform(1.5, 3.0, n)
    instruments = []
    for k in range(nins):
        m = labels == k
        tk = t_all[m]
        tot = np.sqrt(sig[m] ** 2 + cfg['jitters'][k] ** 2)
        if cfg['ma']:
            noise = _ma_noise(rng, tk, tot, cfg['ma']['phi'], cfg['ma']['tau'])
        else:
            noise = rng.normal(0.0, tot)
        yk = rv[m] + cfg['offsets'][k] + noise
        instruments.append(np.column_stack([tk, yk, sig[m]]))
    truth = dict(P=cfg['P'], K=cfg['K'], phase=phase, e=e, w=w, offsets=cfg['offsets'],
                 jitters=cfg['jitters'], ma=cfg['ma'], gp=cfg.get('gp'))
    return instruments, truth


def build_model(name: str, seed: int = 1234, parameterisation: int = 1,
                moav_reference_quirk: bool = False):
    """(ReddModel, RVData, setup, truth-theta) with EMPEROR's default priors.

    Blocks follow ``Simulation._autorun_add_RV_ins`` order (Keplerians first,
    then offset, jitter, MOAV).  Limits are widened where the generating
    values sit outside or on the edge of the defaults (MA coefficient 0.4 >
    0.3 and timescale 5 d on the lower edge of [5, 25], ``block_repo.py:730``);
    each period gets a +-10% search box around its generating value.
    """
    instruments, truth = make_system(name, seed)
    data = preprocess_instruments(instruments, [f'INS{k + 1}' for k in range(len(instruments))])
    ss = SmartSetter(data)
    cfg = CONFIGS[name]
    blocks = []
    for p in range(len(cfg['P'])):
        kb = KeplerianBlock(parameterisation, p + 1)
        ss(kb)
        # period prior around the generating period (a search box, as the
        # reference's tests do with add_condition)
        kb[0].limits = [cfg['P'][p] * 0.9, cfg['P'][p] * 1.1] if parameterisation in (0, 1, 3, 4) \
            else [np.log(cfg['P'][p] * 0.9), np.log(cfg['P'][p] * 1.1)]
        blocks.append(kb)
    ob = OffsetBlock(data.nins)
    ss(ob)
    blocks.append(ob)
    jb = JitterBlock(data.nins)
    ss(jb, jit_prargs=(5, 5))
    blocks.append(jb)
    if cfg['ma']:
        mb = MOAVBlock(data.nins, {'order': cfg['ma']['order'], 'global': False})
        ss(mb)
        for p in mb:
            if p.name.startswith('MACoefficient'):
                p.limits = [0.0, 1.0]
            elif p.name.startswith('MATimescale'):
                p.limits = [1.0, 50.0]
        blocks.append(mb)
    if cfg.get('gp'):
        gb = CeleriteBlock({'terms': ['GonzRotationTerm'],
                            'params': [{'rho': None, 'tau': None, 'A1': None, 'A2': None}]})
        ss(gb)
        # search boxes around the rotation signal, as a user's conditions set them
        for p, lim in zip(gb, ([10.0, 40.0], [10.0, 100.0], [1e-5, 20.0], [1e-5, 20.0])):
            p.limits = lim
        blocks.append(gb)
    model = ReddModel(blocks, data, moav_reference_quirk=moav_reference_quirk)
    theta = truth_theta(model, truth, data, parameterisation)
    return model, data, list(cfg['setup']), theta


def truth_theta(model, truth, data, parameterisation=1):
    """Free-parameter vector at the generating values (offsets shifted by the
    per-instrument mean removal of the preprocessing)."""
    vals = []
    for b in model.blocks:
        if b.type_ == 'Keplerian':
            p = b.number_ - 1
            P, K, ph, e, w = truth['P'][p], truth['K'][p], truth['phase'][p], truth['e'][p], truth['w'][p]
            if parameterisation == 1:
                vals += [P, K, ph, np.sqrt(e) * np.sin(w), np.sqrt(e) * np.cos(w)]
            elif parameterisation == 0:
                vals += [P, K, ph, e, w]
            else:
                raise ValueError('truth only for parameterisations 0/1')
        elif b.type_ == 'Offset':
            vals += [0.0] * len(b)
        elif b.type_ == 'Jitter':
            vals += list(truth['jitters'])
        elif b.type_ == 'MOAV':
            for k in range(len(b) // (2 * b.moav)):
                for c in range(b.moav):
                    vals += [truth['ma']['phi'][c], truth['ma']['tau'][c]]
        elif b.type_ == 'Celerite2':
            g = truth['gp']
            vals += [g['rho'], g['tau'], g['A1'], g['A2']]
    return np.array(vals, dtype=np.float64)


RAGGED = dict(n_systems=4096, n_range=(50, 2000), span=(1000.0, 5000.0), planets=(1, 4),
              P=(1.0, 3000.0), K=(0.5, 100.0), ins=(1, 3), setup=[8, 64, 1000, 1])


def ragged_system(seed: int, s: int):
    """(instruments, truth) of system ``s`` of the ragged batch: its own
    generator keyed by (seed, s), so any subset regenerates identically."""
    cfg = RAGGED
    rng = np.random.default_rng([int(seed), int(s)])
    lo, hi = cfg['n_range']
    n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
    span = rng.uniform(*cfg['span'])
    kp = int(rng.integers(cfg['planets'][0], cfg['planets'][1] + 1))
    nins = int(rng.integers(cfg['ins'][0], cfg['ins'][1] + 1))
    P = np.sort(np.exp(rng.uniform(np.log(cfg['P'][0]), np.log(cfg['P'][1]), kp)))
    K = np.exp(rng.uniform(np.log(cfg['K'][0]), np.log(cfg['K'][1]), kp))
    e = np.minimum(rng.beta(0.87, 3.03, kp), 0.8)
    w = rng.uniform(0, 2 * np.pi, kp)
    phase = rng.uniform(0, 2 * np.pi, kp)
    t = BJD0 + np.sort(rng.uniform(0, span, n))
    tr = t - t[0]
    rv = np.zeros(n)
    for p in range(kp):
        rv += keplerian(tr, P[p], K[p], phase[p], e[p], w[p])
    labels = np.concatenate([np.arange(nins), rng.integers(0, nins, n - nins)])
    rng.shuffle(labels)
    sig = rng.uniform(1.5, 3.0, n)
    offsets = list(rng.uniform(-30, 30, nins))
    jitters = list(rng.uniform(0.5, 3.0, nins))
    instruments = []
    for k in range(nins):
        m = labels == k
        tot = np.sqrt(sig[m] ** 2 + jitters[k] ** 2)
        instruments.append(np.column_stack([t[m], rv[m] + offsets[k] + rng.normal(0.0, tot), sig[m]]))
    truth = dict(P=list(P), K=list(K), phase=list(phase), e=list(e), w=list(w), offsets=offsets,
                 jitters=jitters, ma=None)
    return instruments, truth


def ragged_model(seed: int, s: int):
    """(ReddModel, RVData, truth-theta) of system ``s``: Keplerians
    (parameterisation 1, period box +-10% around the generating period),
    offsets and jitters with EMPEROR's default priors."""
    instruments, truth = ragged_system(seed, s)
    data = preprocess_instruments(instruments, [f'INS{k + 1}' for k in range(len(instruments))])
    ss = SmartSetter(data)
    blocks = []
    for p in range(len(truth['P'])):
        kb = KeplerianBlock(1, p + 1)
        ss(kb)
        kb[0].limits = [truth['P'][p] * 0.9, truth['P'][p] * 1.1]
        blocks.append(kb)
    ob = OffsetBlock(data.nins)
    ss(ob)
    blocks.append(ob)
    jb = JitterBlock(data.nins)
    ss(jb, jit_prargs=(5, 5))
    blocks.append(jb)
    model = ReddModel(blocks, data)
    return model, data, truth_theta(model, truth, data, 1)


def make_ragged(n_systems: int = None, seed: int = 7):
    """[(ReddModel, RVData, truth-theta)] of the ragged batch."""
    n = RAGGED['n_systems'] if n_systems is None else int(n_systems)
    return [ragged_model(seed, s) for s in range(n)]
