"""Model cases shared by the golden-fixture generator and the tests.

Each case builds a model with the package's model layer (the same blocks,
default priors and conditions a Simulation would build) and a fixed,
seeded set of theta: points near the fit, draws inside the limits (some of
which fall outside the derived eccentricity support) and out-of-bounds
points.
"""
from __future__ import annotations

import numpy as np

from astroemperor_gb300.data import preprocess_instruments
from astroemperor_gb300.model import (AccelerationBlock, CeleriteBlock, JitterBlock, KeplerianBlock,
                                      MagneticCycleBlock, MOAVBlock, OffsetBlock, ReddModel,
                                      SinusoidBlock, SmartSetter)
from astroemperor_gb300 import synth

# the 51 Peg fit recorded by the reference (tests/01_51peg_basic.ipynb:548-562)
PEG_MAP_P1 = [4.231, 55.957, 1.769, 0.087, 0.061, 3.642, 2.961]


def peg_data(arr):
    return preprocess_instruments([arr], ['51peg.vels'])


def _kep(ss, par, number, starmass=None, **lims):
    kb = KeplerianBlock(par, number)
    if starmass:
        ss(kb, starmass=starmass, dynamics=True, kplan=number)
    else:
        ss(kb)
    for i, lim in lims.items():
        kb[int(i[1:])].limits = list(lim)
    return kb


def model_51peg(arr, k=1, par=1, conditions=True, fixed_ecc=False, acc=0, moav=None, quirk=False,
                sinusoid=False, cycle=False, gp=None, hill=None):
    data = peg_data(arr)
    ss = SmartSetter(data)
    blocks = []
    if k >= 1:
        if par in (0, 1, 3, 4):
            kb = _kep(ss, par, 1)
            if conditions:
                kb[0].limits = [3, 5]
                kb[1].limits = [45, 60]
        else:
            kb = _kep(ss, par, 1)
            if conditions:
                kb[0].limits = [np.log(3), np.log(5)]
        if par in (3, 4):
            kb[2].limits = [-5, 5]
        if fixed_ecc:
            kb[3].fixed = 0.0
            kb[4].fixed = 0.0
        blocks.append(kb)
    # further Keplerians (inner pairs close enough for the Hill prior to bite)
    for number, plim in ((2, [5.0, 30.0]), (3, [25.0, 150.0]))[:max(0, k - 1)]:
        kb = _kep(ss, par, number, starmass=hill)
        kb[0].limits = plim if par in (0, 1, 3, 4) else [np.log(plim[0]), np.log(plim[1])]
        blocks.append(kb)
    if hill:
        # moderate eccentricities, so that the draws fall on both sides of the
        # Hill criterion rather than mostly past it
        for kb in blocks:
            if kb.parameterisation in (1, 4):
                kb[3].limits = [-0.3, 0.3]
                kb[4].limits = [-0.3, 0.3]
            elif kb.parameterisation in (0, 3):
                kb[3].limits = [0.0, 0.2]
    if sinusoid:
        sb = SinusoidBlock(1)
        ss(sb)
        blocks.append(sb)
    if cycle:
        cb = MagneticCycleBlock(1)
        ss(cb)
        blocks.append(cb)
    if acc:
        ab = AccelerationBlock(acc)
        ss(ab)
        blocks.append(ab)
    ob = OffsetBlock(1)
    ss(ob)
    if conditions:
        ob[0].limits = [-10., 10.]
    blocks.append(ob)
    jb = JitterBlock(1)
    ss(jb, jit_prargs=(5, 5))
    blocks.append(jb)
    if moav:
        mb = MOAVBlock(1, moav)
        ss(mb)
        blocks.append(mb)
    if gp is not None:
        gb = CeleriteBlock(gp)
        ss(gb)
        blocks.append(gb)
    return ReddModel(blocks, data, moav_reference_quirk=quirk), data


# celerite2 kernels of the GP cases: name -> my_kernel (None: free)
GP_KERNELS = {
    'sho_rho_tau_sigma': {'terms': ['SHOTerm'], 'params': [{'rho': None, 'tau': None, 'sigma': None}]},
    'sho_S0_w0_Q': {'terms': ['SHOTerm'], 'params': [{'S0': None, 'w0': None, 'Q': None}]},
    'grot': {'terms': ['GonzRotationTerm'], 'params': [{'rho': None, 'tau': None, 'A1': None, 'A2': None}]},
    'rotation': {'terms': ['RotationTerm'],
                 'params': [{'sigma': None, 'period': None, 'Q0': None, 'dQ': None, 'f': None}]},
    'real_matern': {'terms': ['RealTerm', 'Matern32Term'],
                    'params': [{'a': None, 'c': 0.5}, {'sigma': None, 'rho': None}]},
}


def gp_case_models(arr, n_in=12, n_near=8):
    """name -> (ReddModel, RVData, thetas): 51 Peg, one Keplerian, offset,
    jitter and a celerite2 GP; thetas drawn inside the limits (some past
    the eccentricity support), near the fit with GP amplitudes of a few m/s,
    and out of bounds."""
    rng = np.random.default_rng(20240917)
    out = {}
    for name, ker in GP_KERNELS.items():
        m, d = model_51peg(arr, k=1, par=1, gp=ker)
        free = m.free_parameters()
        lim = m.limits_free()
        c = np.array(PEG_MAP_P1 + [0.0] * (len(free) - len(PEG_MAP_P1)))
        # GP hyperparameters near the middle of their limits
        for j in range(len(PEG_MAP_P1), len(free)):
            c[j] = 0.5 * (lim[j, 0] + lim[j, 1])
        th = draw_thetas(m, rng, n_in=n_in, center=c, n_near=n_near)
        out[name] = (m, d, th)
    # a GP on the residuals of a live MA recurrence: global MA(1), and the
    # documented per-instrument MA(2) (the reference's quirk off)
    for name, ker, moav in (('grot_gma1', GP_KERNELS['grot'], {'order': 1, 'global': True}),
                            ('sho_ma2_inst', GP_KERNELS['sho_rho_tau_sigma'], {'order': 2, 'global': False})):
        m, d = model_51peg(arr, k=1, par=1, gp=ker, moav=moav, quirk=False)
        free = m.free_parameters()
        lim = m.limits_free()
        c = np.array(PEG_MAP_P1 + [0.0] * (len(free) - len(PEG_MAP_P1)))
        for j in range(len(PEG_MAP_P1), len(free)):
            c[j] = 0.5 * (lim[j, 0] + lim[j, 1])
        th = draw_thetas(m, rng, n_in=n_in, center=c, n_near=n_near)
        out[name] = (m, d, th)
    # wider state vectors: two rotation terms (8 dimensions), four
    # GonzRotation terms (16 dimensions)
    rot = {'sigma': None, 'period': None, 'Q0': None, 'dQ': None, 'f': None}
    grot = {'rho': None, 'tau': None, 'A1': None, 'A2': None}
    for name, ker in (('rot_x2', {'terms': ['RotationTerm'] * 2, 'params': [dict(rot), dict(rot)]}),
                      ('grot_x4', {'terms': ['GonzRotationTerm'] * 4, 'params': [dict(grot) for _ in range(4)]})):
        m, d = model_51peg(arr, k=1, par=1, gp=ker)
        free = m.free_parameters()
        lim = m.limits_free()
        c = np.array(PEG_MAP_P1 + [0.0] * (len(free) - len(PEG_MAP_P1)))
        for j in range(len(PEG_MAP_P1), len(free)):
            c[j] = 0.5 * (lim[j, 0] + lim[j, 1])
        th = draw_thetas(m, rng, n_in=n_in, center=c, n_near=n_near)
        out[name] = (m, d, th)
    return out


def draw_thetas(model, rng, n_in=24, center=None, spread=0.02, n_near=8, n_out=4):
    lim = model.limits_free()
    lo, hi = lim[:, 0], lim[:, 1]
    out = [rng.uniform(lo, hi) for _ in range(n_in)]
    if center is not None:
        c = np.asarray(center, dtype=np.float64)
        for _ in range(n_near):
            out.append(c + spread * (hi - lo) * rng.normal(size=len(c)) * 0.1)
    for _ in range(n_out):
        x = rng.uniform(lo, hi)
        i = rng.integers(len(x))
        x[i] = hi[i] + 1.0 + abs(hi[i])
        out.append(x)
    return np.array(out)


def kat_cases(arr):
    """name -> (spec, data dict, thetas [n, ndim])."""
    return {k: (m.spec(), d.as_dict(), th) for k, (m, d, th) in kat_case_models(arr).items()}


def kat_case_models(arr):
    """name -> (ReddModel, RVData, thetas [n, ndim])."""
    rng = np.random.default_rng(20240601)
    cases = {}

    def add(name, model, data, center=None, spread=0.02):
        th = draw_thetas(model, rng, center=center, spread=spread)
        cases[name] = (model, data, th)

    m, d = model_51peg(arr, k=0)
    add('51peg_k0', m, d, center=[3.6, 36.0])
    m, d = model_51peg(arr, k=1, par=1)
    add('51peg_k1_p1', m, d, center=PEG_MAP_P1)
    m, d = model_51peg(arr, k=1, par=0)
    add('51peg_k1_p0', m, d, center=[4.231, 55.957, 1.769, 0.011, 0.964, 3.642, 2.961])
    for par in (2, 3, 4, 6, 7):
        m, d = model_51peg(arr, k=1, par=par)
        add(f'51peg_k1_p{par}', m, d)
    m, d = model_51peg(arr, k=1, par=1, fixed_ecc=True, acc=2)
    add('51peg_fixed_acc', m, d)
    m, d = model_51peg(arr, k=1, par=1, moav={'order': 2, 'global': True})
    add('51peg_gma2', m, d)
    for name, quirk in (('c2_ma1', False), ('c2_ma1_quirk', True)):
        m, d, setup, truth = synth.build_model('c2', seed=7, moav_reference_quirk=quirk)
        add(name, m, d, center=truth)
    # trend blocks: sinusoid00.model and magneticcycle00.model
    m, d = model_51peg(arr, k=1, par=1, sinusoid=True)
    add('51peg_k1_sin', m, d, center=PEG_MAP_P1[:5] + [800.0, 3.0, 1.0] + PEG_MAP_P1[5:])
    m, d = model_51peg(arr, k=1, par=0, cycle=True, moav={'order': 1, 'global': True})
    add('51peg_k1_cycle_gma1', m, d)
    # Hill stability priors (support/priors/Hill.prior) on 2 and 3 Keplerians
    m, d = model_51peg(arr, k=2, par=1, hill=1.11)
    add('51peg_k2_hill', m, d)
    m, d = model_51peg(arr, k=3, par=0, hill=1.11)
    add('51peg_k3_hill_p0', m, d)
    # documented per-instrument MA(2) on one instrument (equal to the
    # reference's live global template on the whole series)
    m, d = model_51peg(arr, k=1, par=1, moav={'order': 2, 'global': False})
    add('51peg_ma2_inst', m, d, center=PEG_MAP_P1 + [0.15, 10.0, 0.1, 12.0])
    # the throughput-scale workload's shape: 7 Keplerians, 4 instruments with
    # documented per-instrument MA(2), N = 16384 over 10000 d (8 epoch tiles
    # of 2048 on the device)
    m, d, setup, truth = synth.build_model('c5', seed=5)
    add('c5_ma2', m, d, center=truth, spread=1e-4)
    # MA(3): the largest order the kernels are built for, global and
    # documented per instrument
    m, d = model_51peg(arr, k=1, par=1, moav={'order': 3, 'global': True})
    add('51peg_gma3', m, d, center=PEG_MAP_P1 + [0.2, 8.0, 0.1, 15.0, 0.05, 30.0])
    m, d = model_51peg(arr, k=1, par=1, moav={'order': 3, 'global': False})
    add('51peg_ma3_inst', m, d, center=PEG_MAP_P1 + [0.2, 8.0, 0.1, 15.0, 0.05, 30.0])
    # real multi-instrument cadence: GJ 876 (eight instruments), two
    # Keplerians; plain, the documented per-instrument MA(1) and the
    # reference's per-instrument MA (a no-op there)
    for name, moav, quirk in (('gj876_k2', None, False),
                              ('gj876_k2_ma1_inst', {'order': 1, 'global': False}, False),
                              ('gj876_k2_ma1_quirk', {'order': 1, 'global': False}, True)):
        m, d = model_gj876(moav=moav, quirk=quirk)
        add(name, m, d, center=gj876_centre(m))
    return cases


def gj876_data():
    """RVData of the GJ 876 fixture (tests/golden/gj876_rv.npz)."""
    import os
    fix = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'gj876_rv.npz'))
    names = [str(n) for n in fix['names']]
    return preprocess_instruments([fix[f'ins_{k}'] for k in range(len(names))], names)


def model_gj876(moav=None, quirk=False):
    """Two parameterisation-1 Keplerians (periods 55-65 d and 28-32 d), an
    offset and a jitter per instrument, optionally per-instrument MA(1)."""
    data = gj876_data()
    ss = SmartSetter(data)
    blocks = []
    for number, plim, klim in ((1, [55.0, 65.0], [150.0, 260.0]), (2, [28.0, 32.0], [40.0, 120.0])):
        kb = _kep(ss, 1, number)
        kb[0].limits = plim
        kb[1].limits = klim
        blocks.append(kb)
    ob = OffsetBlock(data.nins)
    ss(ob)
    blocks.append(ob)
    jb = JitterBlock(data.nins)
    ss(jb, jit_prargs=(5, 5))
    blocks.append(jb)
    if moav:
        mb = MOAVBlock(data.nins, moav)
        ss(mb)
        blocks.append(mb)
    return ReddModel(blocks, data, moav_reference_quirk=quirk), data


# a two-Keplerian maximum of the log posterior of model_gj876() (no MA),
# found with the oracle by Nelder-Mead from a phase grid: P, K, phase,
# sqrt(e) sin w, sqrt(e) cos w of each planet, then the eight offsets and
# the eight jitters (the two inner planets are not modelled, hence ~15 m/s)
GJ876_FIT = [61.0337, 211.906, 6.20890, -3.59882e-04, 9.51621e-04,
             30.2266, 86.9011, 6.28312, 0.0838683, -0.162759,
             -35.6556, 15.2604, 10.6571, 12.8218, 15.8653, 17.5366, 19.7600, -19.8340,
             0.0590557, 14.7155, 14.8289, 15.0750, 15.9099, 15.8155, 13.8305, 14.6368]


def gj876_centre(m):
    """GJ876_FIT, with MA coefficients 0.1 and timescales 5 d, clipped to the limits."""
    lim = m.limits_free()
    c = np.array(GJ876_FIT + [0.1, 5.0] * ((len(lim) - len(GJ876_FIT)) // 2))
    return np.clip(c, lim[:, 0], lim[:, 1])


# ---------------------------------------------------------------------------
# joint RV + astrometry: HIP 21850 (the reference's tests/03_hip21850_test.ipynb)
# ---------------------------------------------------------------------------
# the maximum-posterior fit that notebook recorded (P, K, phase, e, w, I,
# Omega; acceleration; 4 offsets; 4 jitters; 5 astrometric offsets; jitters
# of Hipparcos and Gaia)
HIP_MAP = [2567.37, 120.188, 5.553, 0.201, 0.659, 1.084, 4.289, 0.006,
           -24.341, -4.909, -105.186, -97.556, 29.644, 0.825, 8.933, 1.743,
           -0.437, -0.257, 0.003, -0.183, 0.154, 0.257, 1.086]


def hip21850_data(fix):
    """(RVData, AMData) from the HIP 21850 fixture (tests/golden/hip21850.npz)."""
    from astroemperor_gb300.astrometry import build_am
    names = [str(n) for n in fix['rv_names']]
    inst = [fix[f'rv_{k}'] for k in range(len(names))]
    data = preprocess_instruments(inst, names)
    hg = {k[3:]: fix[k] for k in fix.files if k.startswith('hg_')}
    hipp = {k[5:]: fix[k] for k in fix.files if k.startswith('hipp_')}
    gost = {'ObservationTimeAtBarycentre[BarycentricJulianDateInTCB]': fix['gost_bjd'],
            'scanAngle[rad]': fix['gost_psi'], 'parallaxFactorAlongScan': fix['gost_parf']}
    am = build_am(hg, hipp, gost, fix['dead_dr2'], fix['dead_dr3'], data.common_t)
    return data, am


def model_hip21850(fix, k=1):
    """The notebook's model: one astrometric Keplerian, acceleration, offsets
    and jitters of four instruments, astrometric offsets and jitters, with
    its conditions and prior arguments.  k=2 adds a second astrometric
    Keplerian (periods 20-300 d), a case for the per-planet terms."""
    from astroemperor_gb300.model import (AstrometryJitterBlock, AstrometryKeplerianBlock,
                                          AstrometryOffsetBlock)
    data, am = hip21850_data(fix)
    ss = SmartSetter(data)
    kb = AstrometryKeplerianBlock(1)
    ss(kb, ecc_prargs=(0, 0.3))
    for j, lim in enumerate(([2000, 3000], [50, 150], [np.pi, 2 * np.pi], [0, 0.5], [0, np.pi])):
        kb[j].limits = list(lim)
    kbs = [kb]
    if k == 2:
        kb2 = AstrometryKeplerianBlock(2)
        ss(kb2, ecc_prargs=(0, 0.3))
        for j, lim in enumerate(([20, 300], [1, 30], [0, 2 * np.pi], [0, 0.5], [0, 2 * np.pi])):
            kb2[j].limits = list(lim)
        kbs.append(kb2)
    ab = AccelerationBlock(1)
    ss(ab)
    ob = OffsetBlock(4)
    ss(ob)
    jb = JitterBlock(4)
    ss(jb, jit_prargs=(0, 10))
    for k in range(4):
        ob[k].limits = [-150, 150]
        jb[k].limits = [1e-4, 30]
    aob = AstrometryOffsetBlock()
    ss(aob)
    for p in aob:
        p.limits = [-1, 1]
    ajb = AstrometryJitterBlock()
    ss(ajb)
    ajb[0].limits, ajb[0].prior, ajb[0].prargs = [0, 10], 'Normal', [0, 5]
    ajb[1].limits, ajb[1].prior, ajb[1].prargs = [0, 10], 'Normal', [1, 0.1]
    model = ReddModel(kbs + [ab, ob, jb, aob, ajb], data, am_data=am)
    return model, data, am


# the second planet's (P, K, phase, e, w, I, Omega) around which the k=2 case draws
HIP_K2_PLANET = [97.0, 8.0, 2.0, 0.12, 1.3, 0.9, 2.5]


def am_case_thetas(model, n_in=24, n_near=8):
    rng = np.random.default_rng(20251204)
    center = np.array(HIP_MAP)
    if model.ndim__ == len(HIP_MAP) + 7:
        center = np.concatenate([center[:7], HIP_K2_PLANET, center[7:]])
    return draw_thetas(model, rng, n_in=n_in, center=center, n_near=n_near, spread=0.01)
