"""Model description: parameters, blocks, default priors, and the compiled
device descriptor.

Mirrors the reference's model layer for the blocks on the hot path:

* ``Parameter`` / ``Parameter_Block``  -- ``src/astroemperor/emp_model.py:16-170``
* block factories ``KeplerianBlock``, ``OffsetBlock``, ``JitterBlock``,
  ``MOAVBlock``, ``AccelerationBlock`` -- ``src/astroemperor/block_repo.py:22-240``
* parameter defaults (names, ``is_hou``) -- ``src/astroemperor/param_repo.py:15-180``
* ``SmartSetter`` data-derived limits and priors -- ``block_repo.py:505-868``
* ``ReddModel.refresh__`` theta index maps -- ``emp_model.py:223-330``

Instead of generating Python text for ``my_model``/``my_prior`` the model is
compiled into an ``emp_model_desc`` (``include/emp_gpu.h``) that the CUDA
kernels interpret.
"""
from __future__ import annotations

import copy
import itertools
import math

import numpy as np
from scipy.special import betaln, ndtr

from . import _native as N

# ---------------------------------------------------------------------------
# parameter defaults (param_repo.py)
# ---------------------------------------------------------------------------
_DEFAULTS = {
    'dPeriod': ('Period', False), 'dAmplitude': ('Amplitude', False),
    'dPhase': ('Phase', False), 'dEccentricity': ('Eccentricity', False),
    'dLongitude': ('Longitude', False), 'dlPeriod': ('lPeriod', False),
    'dAmp_sin': ('Amp_sin', True), 'dAmp_cos': ('Amp_cos', True),
    'dEcc_sin': ('Ecc_sin', True), 'dEcc_cos': ('Ecc_cos', True),
    'dT_0': ('T_0', False), 'dM0': ('M0', False),
    'dOffset': ('Offset', False), 'dJitter': ('Jitter', False),
    'dMACoefficient': ('MACoefficient', False), 'dMATimescale': ('MATimescale', False),
    'dAcceleration': ('Acceleration', False),
    # astrometry (param_repo.py:349-445)
    'dInclination': ('Inclination', False), 'dOmega': ('Omega', False),
    'dOffset_ra': ('Offset RA', False), 'dOffset_de': ('Offset DE', False),
    'dOffset_plx': ('Offset PLX', False), 'dOffset_pm_ra': ('Offset pm RA', False),
    'dOffset_pm_de': ('Offset pm DE', False),
    'dJitterH': ('Jitter Hipp', False), 'dJitterG': ('Jitter Gaia', False),
}

# Keplerian parameter lists per parameterisation (block_repo.py:23-31)
KEPLER_PARAMS = {
    0: ['dPeriod', 'dAmplitude', 'dPhase', 'dEccentricity', 'dLongitude'],
    1: ['dPeriod', 'dAmplitude', 'dPhase', 'dEcc_sin', 'dEcc_cos'],
    2: ['dlPeriod', 'dAmp_sin', 'dAmp_cos', 'dEcc_sin', 'dEcc_cos'],
    3: ['dPeriod', 'dAmplitude', 'dT_0', 'dEccentricity', 'dLongitude'],
    4: ['dPeriod', 'dAmplitude', 'dT_0', 'dEcc_sin', 'dEcc_cos'],
    6: ['dlPeriod', 'dAmplitude', 'dPhase', 'dEccentricity', 'dLongitude'],
    7: ['dlPeriod', 'dAmplitude', 'dPhase', 'dEcc_sin', 'dEcc_cos'],
}


class Parameter:
    """One parameter with the reference's attribute names (emp_model.py:16-30)."""

    def __init__(self, key_or_name, **attrs):
        name, is_hou = _DEFAULTS.get(key_or_name, (key_or_name, False))
        self.name = name
        self.prior = 'Uniform'
        self.limits = [None, None]
        self.init_pos = [None, None]
        self.prargs = None
        self.fixed = None
        self.is_hou = is_hou
        self.has_prior = True
        self.has_posterior = True
        self.value = -np.inf
        for k, v in attrs.items():
            setattr(self, k, v)

    def __repr__(self):
        return self.name

    def as_spec(self):
        return {'name': self.name, 'prior': self.prior, 'limits': list(self.limits),
                'prargs': copy.deepcopy(self.prargs), 'fixed': self.fixed,
                'has_prior': self.has_prior}


class Parameter_Block:
    """A block of parameters (emp_model.py:32-170)."""

    def __init__(self, params, **attrs):
        self.list_ = list(params)
        self.additional_parameters = []
        self.parameterisation = None
        self.number_ = 0
        self.moav = 0
        self.is_global = False
        for k, v in attrs.items():
            setattr(self, k, v)
        self.refresh_block()

    def refresh_block(self):
        fixed = [p.fixed for p in self]
        nf = np.array([f is None for f in fixed], dtype=bool)
        self.C_ = np.arange(len(self))[nf]
        self.A_ = np.arange(len(self))[~nf]
        for i in self.A_:
            p = self.list_[i]
            p.value = p.fixed
            p.prior = 'Fixed'
        self.ndim_ = int(nf.sum())

    def get_attr(self, name):
        return [getattr(p, name) for p in self]

    def set_attr(self, name, values):
        for p, v in zip(self, values):
            setattr(p, name, v)

    def __len__(self):
        return len(self.list_)

    def __iter__(self):
        return iter(self.list_)

    def __getitem__(self, i):
        return self.list_[i]

    def __repr__(self):
        return f'{self.name_}({self.ndim_}): {self.list_}'


def KeplerianBlock(parameterisation: int, number: int) -> Parameter_Block:
    """block_repo.py:22-72 (parameterisations 0-4, 6, 7)."""
    if parameterisation not in KEPLER_PARAMS:
        raise ValueError(f'Keplerian parameterisation {parameterisation} is not on this path')
    ps = [Parameter(k) for k in KEPLER_PARAMS[parameterisation]]
    if number:
        for p in ps:
            p.name += f' {number}'
    return Parameter_Block(ps, name_=f'KeplerianBlock {number}', type_='Keplerian',
                           class_='Model', parameterisation=parameterisation, number_=number)


def AstrometryKeplerianBlock(number: int) -> Parameter_Block:
    """block_repo.py:426-448: a parameterisation-0 Keplerian (P, K, phase,
    e, w) with inclination and longitude of the node for the astrometric
    orbit; its RV term is kep00's (akep00.model)."""
    kb = KeplerianBlock(0, number)
    extra = [Parameter(k) for k in ('dInclination', 'dOmega')]
    if number:
        for p in extra:
            p.name += f' {number}'
    kb.list_ = list(kb.list_) + extra
    kb.name_ = f'AstrometryKeplerianBlock {number}'
    kb.astrometry_bool = True
    kb.refresh_block()
    return kb


def AstrometryOffsetBlock() -> Parameter_Block:
    """block_repo.py:451-475: offsets (mas, mas/yr) of the barycentre from
    the Gaia DR3 solution."""
    ps = [Parameter(k) for k in ('dOffset_ra', 'dOffset_de', 'dOffset_plx', 'dOffset_pm_ra',
                                 'dOffset_pm_de')]
    return Parameter_Block(ps, name_='AstrometryOffsetBlock', type_='AstrometryOffset', class_='Data',
                           number_=5)


def AstrometryJitterBlock() -> Parameter_Block:
    """block_repo.py:478-502: jitters of the Hipparcos abscissae and of the
    Gaia catalogue fits."""
    ps = [Parameter(k) for k in ('dJitterH', 'dJitterG')]
    return Parameter_Block(ps, name_='AstrometryJitterBlock', type_='AstrometryJitter', class_='Data',
                           number_=2)


def OffsetBlock(nins: int) -> Parameter_Block:
    """block_repo.py:103-134."""
    ps = []
    for i in range(nins):
        p = Parameter('dOffset')
        p.name += f' {i + 1}'
        ps.append(p)
    return Parameter_Block(ps, name_='OffsetBlock', type_='Offset', class_='Data', number_=nins)


def JitterBlock(nins: int) -> Parameter_Block:
    """block_repo.py:176-203."""
    ps = []
    for i in range(nins):
        p = Parameter('dJitter')
        p.name += f' {i + 1}'
        ps.append(p)
    return Parameter_Block(ps, name_='JitterBlock', type_='Jitter', class_='Data', number_=nins)


def MOAVBlock(nins: int, moav_args: dict) -> Parameter_Block:
    """block_repo.py:206-240: (coefficient, timescale) per instrument and order."""
    order = int(moav_args['order'])
    is_global = bool(moav_args['global'])
    rng = 1 if is_global else nins
    ps = []
    for i, j in itertools.product(range(rng), range(order)):
        pc = Parameter('dMACoefficient')
        pc.name += f' {i + 1} Order {j + 1}'
        pt = Parameter('dMATimescale')
        pt.name += f' {i + 1} Order {j + 1}'
        ps.extend((pc, pt))
    return Parameter_Block(ps, name_='MOAVBlock', type_='MOAV', class_='Data', number_=nins,
                           moav=order, is_global=is_global)


def AccelerationBlock(order: int) -> Parameter_Block:
    """block_repo.py:137-173."""
    ps = []
    for i in range(order):
        p = Parameter('dAcceleration')
        if i > 0:
            p.name = f'Acceleration Order {i + 1}'
        ps.append(p)
    return Parameter_Block(ps, name_=f'AccelerationBlock o{order}', type_='Acceleration',
                           class_='Data', number_=order)


def SinusoidBlock(number: int) -> Parameter_Block:
    """block_repo.py:75-100: A cos(2 pi t / P + phase)."""
    ps = [Parameter(k) for k in ('dPeriod', 'dAmplitude', 'dPhase')]
    if number:
        for p in ps:
            p.name += f' {number}'
    return Parameter_Block(ps, name_='SinusoidBlock', type_='Sinusoid', class_='Model',
                           number_=number)


def MagneticCycleBlock(number: int) -> Parameter_Block:
    """block_repo.py:275-315: A1 cos(pi t / P + phase1) + A2 cos(2 pi t / P + phase2);
    parameter names carry the reference's S1/S2 suffixes."""
    ps = [Parameter(k) for k in ('dPeriod', 'dAmplitude', 'dAmplitude', 'dPhase', 'dPhase')]
    for p, suf in zip(ps, ('S1', 'S1', 'S2', 'S1', 'S2')):
        p.name += f' {suf}'
    return Parameter_Block(ps, name_='MagneticCycleBlock', type_='MagneticCycle', class_='Model',
                           number_=number)


# GP term names of param_repo.py:204-345 by (term, celerite2 keyword)
_GP_NAMES = {'RealTerm': 'Real Term', 'Matern32Term': 'Matern32 Term', 'RotationTerm': 'Rotation Term',
             'SHOTerm': 'SHO Term', 'GonzRotationTerm': 'GRot Term'}
GP_TERMS = tuple(_GP_NAMES)
# terms whose parameters the reference names in a fixed order (block_repo.py:358-370)
# while its kernel text passes the values by the params dictionary's order
# (emp.py:352-366): the i-th parameter takes the i-th name below and the i-th
# dictionary keyword
_GP_FIXED_NAMES = {'RealTerm': ('a', 'c'), 'Matern32Term': ('sigma', 'rho'),
                   'RotationTerm': ('period', 'sigma', 'Q0', 'dQ', 'f')}


def CeleriteBlock(my_kernel: dict) -> Parameter_Block:
    """block_repo.py:350-413: the GP hyperparameters of a celerite2 kernel.

    ``my_kernel = {'terms': ['SHOTerm', ...], 'params': [{'rho': None, 'tau': None,
    'S0': 2.0}, ...]}``: a None value is a free parameter, a number fixes it.
    Parameters follow each term's dictionary order, which is the order in which
    the reference's generated ``my_model`` reads ``theta_gp`` (emp.py:347-370);
    with several terms each name carries the term's 1-based number
    (block_repo.py:393-400).  'GonzRotationTerm' is the reference's two-SHO
    rotation kernel (rho, tau, A1, A2; emp.py:397-412).
    """
    terms, plist = list(my_kernel['terms']), list(my_kernel['params'])
    if len(terms) != len(plist) or not terms:
        raise ValueError('my_kernel needs one params dict per term')
    ps = []
    for t, (term, pd) in enumerate(zip(terms, plist)):
        if term not in _GP_NAMES:
            raise ValueError(f'GP term {term!r} is not built ({", ".join(GP_TERMS)})')
        if term == 'GonzRotationTerm':
            pd = {k: pd.get(k) for k in ('rho', 'tau', 'A1', 'A2')}
        names = list(pd)
        if term in _GP_FIXED_NAMES:
            names = list(_GP_FIXED_NAMES[term])
            if sorted(names) != sorted(pd):
                raise ValueError(f'{term} takes {names}, got {list(pd)}')
        for nm, (k, v) in zip(names, pd.items()):
            p = Parameter(f'{_GP_NAMES[term]} {nm}' + (str(t + 1) if len(terms) > 1 else ''))
            p.gp_term, p.gp_key = t, k
            if v is not None:
                p.fixed = float(v)
            ps.append(p)
    return Parameter_Block(ps, name_='CeleriteBlock', type_='Celerite2', class_='Model',
                           number_=len(terms), my_kernel={'terms': terms, 'params': plist})


class SmartSetter:
    """Data-derived default limits and priors (block_repo.py:505-868)."""

    def __init__(self, data):
        self.data = data
        self.angular = [0, 2 * np.pi]

    def _amp_per(self):
        sig = float(np.std(self.data.RV))            # pandas std(ddof=0)
        per = float(self.data.BJD.max() - self.data.BJD.min())
        return sig * np.sqrt(4), per

    def set_Keplerian(self, b, ecc_limits=(0, 1), ecc_prargs=(0, 0.1), starmass=None, dynamics=False,
                      kplan=None, dynamics_already_included=False):
        amp, per = self._amp_per()
        uni = 'Uniform'
        par = b.parameterisation
        add_ecc = False
        ecc_extra_prargs = None
        if par == 0:
            lims = [[1.5, per], [1e-6, amp], self.angular, list(ecc_limits), self.angular]
            priors = [uni, uni, uni, 'Normal', uni]
            prargs = [None, None, None, list(ecc_prargs), None]
            if getattr(b, 'astrometry_bool', False):
                # inclination (isotropic) and node (block_repo.py:534-537)
                lims += [[0, np.pi], list(self.angular)]
                priors += ['Isotropic', uni]
                prargs += [None, None]
        elif par == 1:
            lims = [[1.5, per], [1e-6, amp], self.angular, [-1, 1], [-1, 1]]
            priors, prargs = [uni] * 5, [None] * 5
            add_ecc = True
        elif par == 2:
            kamp = np.sqrt(amp / 2)
            lims = [[np.log(1.5), np.log(per)], [-kamp, kamp], [-kamp, kamp], [-1, 1], [-1, 1]]
            priors, prargs = [uni] * 5, [None] * 5
            add_ecc = True
        elif par == 3:
            lims = [[1.5, per], [1e-6, amp], [-1000, 1000], list(ecc_limits), self.angular]
            priors = [uni, uni, uni, 'Normal', uni]
            prargs = [None, None, None, list(ecc_prargs), None]
        elif par == 4:
            lims = [[1.5, per], [1e-6, amp], [-1000, 1000], [-1, 1], [-1, 1]]
            priors, prargs = [uni] * 5, [None] * 5
            add_ecc = True
        elif par == 6:
            lims = [[np.log(1.5), np.log(per)], [1e-6, amp], self.angular, list(ecc_limits), self.angular]
            priors = ['Jeffreys', uni, uni, 'Normal', uni]
            prargs = [None, None, None, list(ecc_prargs), None]
        elif par == 7:
            lims = [[np.log(1.5), np.log(per)], [1e-6, amp], self.angular, [-1, 1], [-1, 1]]
            priors = ['Jeffreys', uni, uni, uni, uni]
            prargs = [None] * 5
            add_ecc = True
            ecc_extra_prargs = list(ecc_prargs)
        else:
            raise ValueError(par)
        if add_ecc:   # ecc_w_add_additional (block_repo.py:666-688)
            e = Parameter('dEccentricity', has_prior=True, limits=[0, 1])
            if ecc_extra_prargs is not None:
                e.prior = 'Normal'
                e.prargs = ecc_extra_prargs
            w = Parameter('dLongitude', has_prior=False, limits=list(self.angular))
            for ap in (e, w):
                if b.number_:
                    ap.name += f' {b.number_}'
            b.additional_parameters = [e, w]
        kplan = b.number_ if kplan is None else kplan
        if starmass and dynamics and not dynamics_already_included and kplan > 1:
            # block_repo.py:611-626: a Hill prior over the first kplan planets
            b.additional_parameters = list(b.additional_parameters) + [
                Parameter('Hill', prior='Hill', limits=[None, None], prargs=[int(kplan), float(starmass)],
                          has_prior=True, has_posterior=False)]
        return lims, priors, prargs

    def _per_ins_absmax(self, b):
        out = []
        for nin in range(b.number_):
            m = self.data.Flag == (nin + 1)
            out.append(float(np.max(np.abs(self.data.RV[m]))))
        return out

    def set_Offset(self, b, **kw):
        lims = [[-a, a] for a in self._per_ins_absmax(b)]
        return lims, ['Uniform'] * len(lims), [None] * len(lims)

    def set_Jitter(self, b, jit_prargs=(5, 5), **kw):
        lims = [[1e-5, a] for a in self._per_ins_absmax(b)]
        return lims, ['Normal'] * len(lims), [list(jit_prargs) for _ in lims]

    def set_MOAV(self, b, **kw):
        lims, priors, prargs = [], [], []
        n = 1 if b.is_global else b.number_
        for _ in range(n):
            for _ in range(b.moav):
                lims += [[0.0, 0.3], [5, 25]]
                priors += ['Uniform', 'Uniform']
                prargs += [None, None]
        return lims, priors, prargs

    def set_Sinusoid(self, b, **kw):
        """block_repo.py:805-817."""
        amp, per = self._amp_per()
        lims = [[1.5, per], [1e-6, amp], list(self.angular)]
        return lims, ['Uniform'] * 3, [None] * 3

    def set_MagneticCycle(self, b, **kw):
        """block_repo.py:819-833."""
        amp, per = self._amp_per()
        lims = [[1.5, per], [1e-6, amp], [1e-6, amp], list(self.angular), list(self.angular)]
        return lims, ['Uniform'] * 5, [None] * 5

    def set_Celerite2(self, b, **kw):
        """block_repo.py:761-790: free hyperparameters Uniform in [1e-5, 5]
        ([1e-5, 1] for the RotationTerm mixing fraction f)."""
        lims = [[1e-5, 1.0] if p.gp_key == 'f' else [1e-5, 5.0] for p in b]
        return lims, ['Uniform' if p.fixed is None else 'Fixed' for p in b], [None] * len(lims)

    def set_AstrometryOffset(self, b, **kw):
        """block_repo.py:843-850."""
        return [[-1e1, 1e1]] * 5, ['Uniform'] * 5, [None] * 5

    def set_AstrometryJitter(self, b, **kw):
        """block_repo.py:835-840 (Hipparcos, Gaia)."""
        return [[0, 20], [0, 10]], ['Uniform', 'Uniform'], [None, None]

    def set_Acceleration(self, b, **kw):
        return [[-1, 1]] * b.number_, ['Uniform'] * b.number_, [None] * b.number_

    def __call__(self, block, **kw):
        lims, priors, prargs = getattr(self, f'set_{block.type_}')(block, **kw)
        block.set_attr('limits', [list(l) for l in lims])
        block.set_attr('prior', priors)
        block.set_attr('prargs', prargs)


# ---------------------------------------------------------------------------
# prior arguments (emp_model.py:82-120)
# ---------------------------------------------------------------------------
def prior_struct(prior: str, limits, prargs) -> N.EmpPrior:
    """One compiled prior; the normalisers follow ``_check_prargs``."""
    p = N.EmpPrior()
    if prior in (None, 'None'):
        p.kind = N.EMP_PRIOR_NONE
        return p
    if prior not in N.PRIOR_KIND:
        raise ValueError(f'prior {prior!r} is not on this path '
                         '(Uniform, Normal, Jeffreys, Beta, Isotropic, Fixed)')
    low, high = float(limits[0]), float(limits[1])
    p.kind = N.PRIOR_KIND[prior]
    p.lo, p.hi = low, high
    if prior in ('Uniform', 'Jeffreys'):
        p.a0 = float(np.log(1 / (high - low)))
    elif prior == 'Isotropic':
        # log(sin(x) / 2) - logZ, logZ = log((cos lo - cos hi) / 2) (emp_model.py:96-99)
        p.a0 = float(np.log(0.5 * (np.cos(low) - np.cos(high))))
    elif prior == 'Normal':
        mu, s = float(prargs[0]), float(prargs[1])
        a, b = (low - mu) / s, (high - mu) / s
        logZ = float(np.log(ndtr(b) - ndtr(a)))
        p.a0, p.a1 = mu, 1.0 / s          # the device multiplies by 1/s
        p.a2 = float(np.log(s * np.sqrt(2 * np.pi))) + logZ
    elif prior == 'Beta':
        a, b = float(prargs[0]), float(prargs[1])
        p.a0, p.a1, p.a2 = a, b, float(betaln(a, b))
    return p


class ReddModel:
    """The run's model: blocks, theta layout, spec and device descriptor.

    Restates ``ReddModel.refresh__`` (emp_model.py:223-330): global slices,
    free (``C_``) and fixed (``A_``) index maps, ``ndim__``.
    """

    HOT_TYPES = ('Keplerian', 'Acceleration', 'Offset', 'Jitter', 'MOAV', 'Sinusoid', 'MagneticCycle',
                 'Celerite2', 'AstrometryOffset', 'AstrometryJitter')

    def __init__(self, blocks, data, moav_reference_quirk=False, am_data=None):
        self.blocks = list(blocks)
        self.data = data
        self.moav_reference_quirk = bool(moav_reference_quirk)
        # astrometric data (astrometry.AMData) of a joint fit, with the
        # AstrometryOffset / AstrometryJitter blocks
        self.am_data = am_data
        self.refresh__()

    def __iter__(self):
        return iter(self.blocks)

    def refresh__(self):
        blen = 0
        self.ndim__ = 0
        for b in self.blocks:
            if b.type_ not in self.HOT_TYPES:
                raise ValueError(f'block type {b.type_} is not on the GPU hot path')
            b.refresh_block()
            b.slice = slice(blen, blen + len(b))
            blen += len(b)
            self.ndim__ += b.ndim_
        self.n_full = blen
        fixed = [p.fixed for b in self.blocks for p in b]
        free = np.array([f is None for f in fixed], dtype=bool)
        self.C_ = np.arange(blen)[free]
        self.A_ = np.arange(blen)[~free]
        self.mod_fixed = np.array(fixed, dtype=object)
        self.kplan__ = sum(1 for b in self.blocks if b.type_ == 'Keplerian')
        self.nins__ = self.data.nins
        gp = [b for b in self.blocks if b.type_ == 'Celerite2']
        if len(gp) > 1:
            raise ValueError('one Celerite2 block per model')
        # with a live MOAV block the GP models the residuals after the MA
        # recurrence (02.like: gp_.mean = my_model's model, which the MA terms
        # are part of); the reference's per-instrument MOAV is a no-op
        # (moav00.model:18-19), so with the quirk the GP sees the plain residuals
        am = [b for b in self.blocks if b.type_ in ('AstrometryOffset', 'AstrometryJitter')]
        if am:
            types = sorted(b.type_ for b in am)
            if types != ['AstrometryJitter', 'AstrometryOffset']:
                raise ValueError('astrometry needs one AstrometryOffset and one AstrometryJitter block')
            if self.am_data is None:
                raise ValueError('astrometry blocks without astrometric data (am_data)')
            if gp:
                raise ValueError('a GP likelihood and astrometry cannot be combined on this path')
            for b in self.blocks:
                if b.type_ == 'Keplerian' and not getattr(b, 'astrometry_bool', False):
                    raise ValueError('with astrometry every Keplerian is an AstrometryKeplerianBlock')
        # the MOAV residual is taken after every mean-model block
        seen_moav = False
        for b in self.blocks:
            if b.type_ == 'MOAV':
                seen_moav = True
            elif seen_moav and b.type_ in ('Keplerian', 'Acceleration', 'Offset', 'Sinusoid',
                                           'MagneticCycle'):
                raise ValueError('MOAV block must follow the Keplerian, sinusoid, magnetic-cycle, '
                                 'acceleration and offset blocks')

    # plain dict spec (used by the CPU oracle in tests)
    def spec(self) -> dict:
        out = []
        for b in self.blocks:
            d = {'type': b.type_, 'params': [p.as_spec() for p in b]}
            if b.type_ == 'Keplerian':
                d['parameterisation'] = b.parameterisation
                d['additional'] = [p.as_spec() for p in b.additional_parameters]
                if getattr(b, 'astrometry_bool', False):
                    d['astrometry'] = True
            if b.type_ == 'MOAV':
                d['order'] = b.moav
                d['global'] = b.is_global
            if b.type_ == 'Celerite2':
                d['gp_terms'] = self.gp_terms()
            out.append(d)
        return {'nins': self.nins__, 'blocks': out,
                'moav_reference_quirk': self.moav_reference_quirk}

    def gp_terms(self):
        """[(kind, [full-theta slot of each canonical parameter])] of the
        Celerite2 block (kinds and canonical orders of oracle.gp / EMP_GP_*)."""
        out = []
        for b in self.blocks:
            if b.type_ != 'Celerite2':
                continue
            for t, term in enumerate(b.my_kernel['terms']):
                slot = {p.gp_key: b.slice.start + i for i, p in enumerate(b) if p.gp_term == t}
                keys = tuple(slot)
                if term == 'SHOTerm':
                    amp = 'sigma' if 'sigma' in slot else 'S0'
                    freq = 'rho' if 'rho' in slot else 'w0'
                    qual = 'tau' if 'tau' in slot else 'Q'
                    if {amp, freq, qual} != set(keys):
                        raise ValueError(f'SHOTerm keywords {sorted(keys)} are not (S0|sigma, w0|rho, Q|tau)')
                    kind = N.EMP_GP_SHO + (amp == 'sigma') + 2 * (freq == 'rho') + 4 * (qual == 'tau')
                    order = (amp, freq, qual)
                else:
                    kind, order = {'RealTerm': (N.EMP_GP_REAL, ('a', 'c')),
                                   'Matern32Term': (N.EMP_GP_MATERN32, ('sigma', 'rho')),
                                   'RotationTerm': (N.EMP_GP_ROTATION, ('sigma', 'period', 'Q0', 'dQ', 'f')),
                                   'GonzRotationTerm': (N.EMP_GP_GROT, ('rho', 'tau', 'A1', 'A2'))}[term]
                    if set(order) != set(keys):
                        raise ValueError(f'{term} takes {order}, got {keys}')
                out.append((kind, [slot[k] for k in order]))
        return out

    def free_parameters(self):
        return [p for b in self.blocks for p in b if p.fixed is None]

    def limits_free(self) -> np.ndarray:
        return np.array([list(map(float, p.limits)) for p in self.free_parameters()])

    def descriptor(self) -> N.EmpModelDesc:
        """Compile to ``emp_model_desc``."""
        if self.n_full > N.EMP_MAX_PARAMS:
            raise ValueError(f'{self.n_full} parameters exceed {N.EMP_MAX_PARAMS}')
        md = N.EmpModelDesc()
        md.abi_version = N.EMP_ABI_VERSION
        md.n_full = self.n_full
        md.n_free = self.ndim__
        md.n_ins = self.nins__
        md.offset_slot = md.jitter_slot = md.ma_slot = md.acc_slot = -1
        md.am_offset_slot = md.am_jitter_slot = -1
        planet = 0
        free_i = 0
        for b in self.blocks:
            s0 = b.slice.start
            if b.type_ == 'Keplerian':
                if planet >= N.EMP_MAX_PLANETS:
                    raise ValueError('too many Keplerians')
                md.kep_param[planet] = b.parameterisation
                md.kep_slot[planet] = s0
                md.derived[planet][0] = prior_struct('None', None, None)
                md.derived[planet][1] = prior_struct('None', None, None)
                for ap in b.additional_parameters:
                    if not getattr(ap, 'has_prior', False):
                        continue
                    if ap.name == 'Hill':
                        j = int(ap.prargs[0])
                        if j > 1:                             # emp.py:222
                            if j > N.EMP_MAX_PLANETS:
                                raise ValueError(f'Hill prior over {j} planets')
                            if md.hill_mask and md.hill_starmass != float(ap.prargs[1]):
                                raise ValueError('Hill priors with different star masses')
                            md.hill_mask |= 1 << j
                            md.hill_starmass = float(ap.prargs[1])
                    elif ap.name[:3] == 'Ecc':
                        md.derived[planet][0] = prior_struct(ap.prior, ap.limits, ap.prargs)
                    elif ap.name[:3] == 'Amp':
                        md.derived[planet][1] = prior_struct(ap.prior, ap.limits, ap.prargs)
                planet += 1
            elif b.type_ in ('Sinusoid', 'MagneticCycle'):
                # cosine terms: e = 0 Keplerian terms of the kernel (kinds 8, 9, 10)
                kinds = (N.EMP_TERM_SINUSOID,) if b.type_ == 'Sinusoid' else (N.EMP_TERM_CYCLE_1, N.EMP_TERM_CYCLE_2)
                for kind in kinds:
                    if planet >= N.EMP_MAX_PLANETS:
                        raise ValueError('too many Keplerian and cosine terms')
                    md.kep_param[planet] = kind
                    md.kep_slot[planet] = s0
                    md.derived[planet][0] = prior_struct('None', None, None)
                    md.derived[planet][1] = prior_struct('None', None, None)
                    planet += 1
            elif b.type_ == 'Celerite2':
                pass                                          # gp_terms below
            elif b.type_ == 'Offset':
                md.offset_slot = s0
            elif b.type_ == 'Jitter':
                md.jitter_slot = s0
            elif b.type_ == 'MOAV':
                if b.moav > N.EMP_MAX_MA:
                    raise ValueError(f'MA order {b.moav} > {N.EMP_MAX_MA}')
                md.ma_slot = s0
                md.ma_order = b.moav
                md.ma_global = int(b.is_global)
                md.ma_quirk = int(self.moav_reference_quirk)
            elif b.type_ == 'Acceleration':
                md.acc_slot = s0
                md.acc_order = len(b)
            elif b.type_ == 'AstrometryOffset':
                md.am_on = 1
                md.am_offset_slot = s0
            elif b.type_ == 'AstrometryJitter':
                md.am_jitter_slot = s0
            for i, p in enumerate(b):
                slot = s0 + i
                if p.fixed is None:
                    md.full_src[slot] = free_i
                    md.full_fixed[slot] = 0.0
                    md.prior_slot[free_i] = slot
                    if p.prior == 'Fixed':
                        raise ValueError(f'{p.name}: free parameter with a Fixed prior')
                    md.prior[free_i] = prior_struct(p.prior, p.limits, p.prargs)
                    free_i += 1
                else:
                    md.full_src[slot] = -1
                    md.full_fixed[slot] = float(p.fixed)
        md.n_planets = planet
        gpt = self.gp_terms()
        if len(gpt) > N.EMP_MAX_GP_TERMS:
            raise ValueError(f'{len(gpt)} GP terms exceed {N.EMP_MAX_GP_TERMS}')
        md.gp_nterms = len(gpt)
        for k, (kind, slots) in enumerate(gpt):
            md.gp_kind[k] = kind
            for i in range(5):
                md.gp_slot[k][i] = slots[i] if i < len(slots) else -1
        md.loglike_const = float(- 0.5 * np.log(2 * np.pi) * self.data.ndata)
        # constant prior terms summed in my_prior's order (block by block,
        # each Keplerian block followed by its derived priors)
        const, var = 0.0, []
        planet = 0
        fi = 0
        for b in self.blocks:
            for p in b:
                if p.fixed is not None:
                    continue
                pr = md.prior[fi]
                if pr.kind in (N.PRIOR_KIND['Uniform'], N.PRIOR_KIND['Jeffreys']):
                    const += pr.a0
                else:
                    var.append(fi)
                fi += 1
            if b.type_ == 'Keplerian':
                for k in range(2):
                    pr = md.derived[planet][k]
                    if pr.kind in (N.PRIOR_KIND['Uniform'], N.PRIOR_KIND['Jeffreys']):
                        const += pr.a0
                    elif pr.kind != N.EMP_PRIOR_NONE:
                        var.append(self.ndim__ + 2 * planet + k)
                planet += 1
        md.prior_const = float(const)
        md.n_prior_var = len(var)
        for i, v in enumerate(var):
            md.prior_var[i] = v
        return md


def full_theta(model: ReddModel, theta):
    """np.insert of the fixed values (emp_model.py:709-711) for a batch."""
    theta = np.atleast_2d(np.asarray(theta, dtype=np.float64))
    out = np.empty((theta.shape[0], model.n_full))
    out[:, model.C_] = theta
    for a in model.A_:
        out[:, a] = float(model.mod_fixed[a])
    return out


def normal_logZ(low, high, mu, s) -> float:
    """ln(Phi(b) - Phi(a)) of a truncated normal (emp_model.py:90-94)."""
    a, b = (low - mu) / s, (high - mu) / s
    return math.log(ndtr(b) - ndtr(a))
