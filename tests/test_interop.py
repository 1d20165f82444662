"""Adapter from the reference's block objects (duck-typed stand-ins)."""
from types import SimpleNamespace

import numpy as np

from astroemperor_gb300.interop import data_from_frame, model_from_blocks
from oracle.rv import OracleRV, check_prargs
from tests.golden.cases import model_51peg


def _ref_like(block, normalise=True):
    """A stand-in with the attributes of the reference's Parameter_Block after
    refresh__ (prargs replaced by their normalised form, emp_model.py:82-98)."""
    ps = []
    for p in block:
        pr = p.prargs
        if normalise:
            pr = check_prargs(p.prior, p.limits, p.prargs)
        ps.append(SimpleNamespace(name=p.name, prior=p.prior, limits=list(p.limits), prargs=pr,
                                  fixed=p.fixed, init_pos=list(p.init_pos), is_hou=p.is_hou))
    extra = [SimpleNamespace(name=a.name, prior=a.prior, limits=list(a.limits),
                             prargs=check_prargs(a.prior, a.limits, a.prargs), has_prior=a.has_prior)
             for a in getattr(block, 'additional_parameters', [])]

    class B(list):
        pass
    b = B(ps)
    b.type_ = block.type_
    b.parameterisation = block.parameterisation
    b.number_ = block.number_
    b.moav = block.moav
    b.is_global = block.is_global
    b.additional_parameters = extra
    b.astrometry_bool = getattr(block, 'astrometry_bool', False)
    return b


def test_model_from_reference_blocks(peg_arr):
    m, d = model_51peg(peg_arr, k=1, par=1, moav={'order': 1, 'global': True})
    frame = {'BJD': d.BJD, 'RV': d.RV, 'eRV': d.eRV, 'Flag': d.Flag}
    d2 = data_from_frame(frame, common_t=d.common_t)
    m2 = model_from_blocks([_ref_like(b) for b in m.blocks], d2)
    a, b = m.descriptor(), m2.descriptor()
    assert bytes(a) == bytes(b)
    o = OracleRV(m2.spec(), d2.as_dict())
    th = np.array([4.231, 55.957, 1.769, 0.087, 0.061, 3.642, 2.961, 0.1, 10.0])
    assert np.isfinite(o.my_prior(th)) and np.isfinite(o.my_likelihood(th))


def test_model_with_gp_from_reference_blocks(peg_arr):
    from tests.golden.cases import GP_KERNELS
    ker = GP_KERNELS['real_matern']
    m, d = model_51peg(peg_arr, k=1, par=1, gp=ker)
    frame = {'BJD': d.BJD, 'RV': d.RV, 'eRV': d.eRV, 'Flag': d.Flag}
    d2 = data_from_frame(frame, common_t=d.common_t)
    m2 = model_from_blocks([_ref_like(b) for b in m.blocks], d2, my_kernel=ker)
    assert bytes(m.descriptor()) == bytes(m2.descriptor())
    import pytest
    with pytest.raises(ValueError, match='my_kernel'):
        model_from_blocks([_ref_like(b) for b in m.blocks], d2)


def test_rotation_term_names_follow_the_reference():
    # names in the reference's fixed order, values by the dictionary's order
    from astroemperor_gb300.model import CeleriteBlock
    b = CeleriteBlock({'terms': ['RotationTerm'],
                       'params': [{'sigma': None, 'period': None, 'Q0': None, 'dQ': None, 'f': None}]})
    assert [p.name for p in b] == ['Rotation Term period', 'Rotation Term sigma', 'Rotation Term Q0',
                                   'Rotation Term dQ', 'Rotation Term f']
    assert [p.gp_key for p in b] == ['sigma', 'period', 'Q0', 'dQ', 'f']


def test_model_with_hill_from_reference_blocks(peg_arr):
    m, d = model_51peg(peg_arr, k=3, par=1, hill=1.11)
    frame = {'BJD': d.BJD, 'RV': d.RV, 'eRV': d.eRV, 'Flag': d.Flag}
    d2 = data_from_frame(frame, common_t=d.common_t)
    m2 = model_from_blocks([_ref_like(b) for b in m.blocks], d2)
    assert bytes(m.descriptor()) == bytes(m2.descriptor())
    assert m2.descriptor().hill_mask == (1 << 2) | (1 << 3)


def test_model_with_astrometry_from_reference_blocks():
    """The HIP 21850 model (tests/03_hip21850_test.ipynb) from stand-ins of the
    reference's blocks compiles to the same descriptor and likelihood."""
    import os
    from tests.golden.cases import HIP_MAP, model_hip21850
    fix = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'hip21850.npz'))
    m, d, am = model_hip21850(fix)
    frame = {'BJD': d.BJD, 'RV': d.RV, 'eRV': d.eRV, 'Flag': d.Flag}
    d2 = data_from_frame(frame, labels=d.labels, common_t=d.common_t)
    m2 = model_from_blocks([_ref_like(b) for b in m.blocks], d2, am_data=am)
    assert bytes(m.descriptor()) == bytes(m2.descriptor())
    o1 = OracleRV(m.spec(), dict(d.as_dict(), am=am.as_dict()))
    o2 = OracleRV(m2.spec(), dict(d2.as_dict(), am=am.as_dict()))
    x = np.array(HIP_MAP)
    assert o1.my_likelihood(x) == o2.my_likelihood(x)
    assert o1.my_prior(x) == o2.my_prior(x)
