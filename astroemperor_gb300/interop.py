"""Adapters from EMPEROR's own objects to this package.

A maintainer who wires the GPU engine into EMPEROR hands it the reference's
``Parameter_Block`` list (``self.model`` after ``update_model``,
``emp.py:2391-2399``) and its ``my_data`` DataFrame (columns BJD, RV, eRV,
Flag, already preprocessed by ``DataWrapper.get_data__``).  The blocks are
read by attribute only (duck typing), so this module needs neither pandas
nor the reference installed.
"""
from __future__ import annotations

import numpy as np

from .data import RVData
from .model import (AccelerationBlock, AstrometryJitterBlock, AstrometryKeplerianBlock, AstrometryOffsetBlock,
                    CeleriteBlock, JitterBlock, KeplerianBlock, MagneticCycleBlock, MOAVBlock, OffsetBlock,
                    Parameter, ReddModel, SinusoidBlock)


def data_from_frame(df, labels=None, common_t=0.0) -> RVData:
    """RVData from a table with BJD, RV, eRV, Flag columns (already referenced)."""
    bjd = np.asarray(df['BJD'], dtype=np.float64)
    order = np.argsort(bjd, kind='mergesort')
    flag = np.asarray(df['Flag'], dtype=np.int64)[order]
    nins = int(flag.max())
    return RVData(BJD=bjd[order], RV=np.asarray(df['RV'], dtype=np.float64)[order],
                  eRV=np.asarray(df['eRV'], dtype=np.float64)[order], Flag=flag,
                  common_t=float(common_t),
                  labels=list(labels) if labels else [f'INS{k + 1}' for k in range(nins)])


def _copy_params(src_block, dst_block):
    for ps, pd in zip(src_block, dst_block):
        for attr in ('name', 'prior', 'limits', 'prargs', 'fixed', 'init_pos', 'is_hou'):
            if hasattr(ps, attr):
                setattr(pd, attr, getattr(ps, attr))
        # the reference stores normalised prargs ([mu, s, logZ] / logZ) after
        # refresh__; the compiler recomputes the normalisers from (mu, s)
        if pd.prior == 'Normal' and pd.prargs is not None:
            pd.prargs = list(pd.prargs)[:2]
        elif pd.prior in ('Uniform', 'Jeffreys'):
            pd.prargs = None
    return dst_block


def model_from_blocks(blocks, data: RVData, moav_reference_quirk=False, my_kernel=None,
                      am_data=None) -> ReddModel:
    """ReddModel from the reference's block list (emp_model.py:32-170 objects).

    A 'Celerite2' block needs the Simulation's ``my_kernel`` (the reference's
    block does not keep it; emp.py:1283-1296 builds it from ``self.my_kernel``).
    A joint RV + astrometry model (Keplerian blocks with ``astrometry_bool``,
    'AstrometryOffset' and 'AstrometryJitter' blocks) needs the astrometric
    data: ``astrometry.load_am`` on the same ``datafiles/<star>/AM/`` folder
    the reference read.
    """
    out = []
    for b in blocks:
        t = b.type_
        if t == 'Keplerian' and getattr(b, 'astrometry_bool', False):
            nb = AstrometryKeplerianBlock(int(b.number_))
        elif t == 'AstrometryOffset':
            nb = AstrometryOffsetBlock()
        elif t == 'AstrometryJitter':
            nb = AstrometryJitterBlock()
        elif t == 'Keplerian':
            nb = KeplerianBlock(int(b.parameterisation), int(b.number_))
            extra = []
            for ap in getattr(b, 'additional_parameters', []):
                p = Parameter(getattr(ap, 'name', 'extra'))
                for attr in ('name', 'prior', 'limits', 'prargs', 'has_prior'):
                    if hasattr(ap, attr):
                        setattr(p, attr, getattr(ap, attr))
                if p.prior == 'Normal' and p.prargs is not None:
                    p.prargs = list(p.prargs)[:2]
                extra.append(p)
            nb.additional_parameters = extra
        elif t == 'Offset':
            nb = OffsetBlock(len(b))
        elif t == 'Jitter':
            nb = JitterBlock(len(b))
        elif t == 'MOAV':
            nb = MOAVBlock(int(b.number_), {'order': int(b.moav), 'global': bool(b.is_global)})
        elif t == 'Acceleration':
            nb = AccelerationBlock(len(b))
        elif t == 'Sinusoid':
            nb = SinusoidBlock(int(b.number_))
        elif t == 'MagneticCycle':
            nb = MagneticCycleBlock(int(b.number_))
        elif t == 'Celerite2':
            if my_kernel is None:
                raise ValueError('a Celerite2 block needs my_kernel (Simulation.my_kernel)')
            nb = CeleriteBlock(my_kernel)
        else:
            raise ValueError(f'block type {t!r} is not on the GPU hot path')
        out.append(_copy_params(b, nb))
    # the reference appends sinusoid and magnetic-cycle blocks after the MOAV
    # block (emp.py:2633-2650).  Its per-instrument MOAV is a no-op, so with
    # the reference quirk the order does not matter and the cosine blocks move
    # ahead of it; with a live MA the model is rejected by ReddModel.
    ma = [i for i, b in enumerate(out) if b.type_ == 'MOAV']
    if ma and moav_reference_quirk and not out[ma[0]].is_global:
        cos = [b for b in out[ma[0]:] if b.type_ in ('Sinusoid', 'MagneticCycle')]
        rest = [b for b in out if b not in cos]
        k = next(i for i, b in enumerate(rest) if b.type_ == 'MOAV')
        out = rest[:k] + cos + rest[k:]
    return ReddModel(out, data, moav_reference_quirk=moav_reference_quirk, am_data=am_data)
