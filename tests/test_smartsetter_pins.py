"""Default limits, priors and prior arguments of every block type against the
reference's own SmartSetter methods (tests/golden/smartsetter_kat.json, written
by tests/golden/make_golden.py from block_repo.py's source)."""
import json

import numpy as np
import pytest

from astroemperor_gb300 import synth
from astroemperor_gb300.model import (AccelerationBlock, JitterBlock, KeplerianBlock, MagneticCycleBlock,
                                      MOAVBlock, OffsetBlock, SinusoidBlock, SmartSetter)
from tests.golden.cases import peg_data

KAT = json.load(open('tests/golden/smartsetter_kat.json'))


def _data(name, peg_arr):
    if name == '51peg':
        return peg_data(peg_arr)
    return synth.build_model('c2', seed=1234)[1]


def _blocks(nins):
    out = {f'Keplerian{p}': (KeplerianBlock(p, 1), dict(ecc_limits=(0, 1), ecc_prargs=(0, 0.1)))
           for p in (0, 1, 2, 3, 4, 6, 7)}
    out.update({
        'Offset': (OffsetBlock(nins), {}),
        'Jitter': (JitterBlock(nins), dict(jit_prargs=(5, 5))),
        'MOAV2': (MOAVBlock(nins, {'order': 2, 'global': False}), {}),
        'Acceleration2': (AccelerationBlock(2), {}),
        'Sinusoid': (SinusoidBlock(1), {}),
        'MagneticCycle': (MagneticCycleBlock(1), {}),
    })
    return out


@pytest.mark.parametrize('dname', ['51peg', 'c2'])
def test_smartsetter_equals_reference(peg_arr, dname):
    d = _data(dname, peg_arr)
    ss = SmartSetter(d)
    for key, (b, kw) in _blocks(d.nins).items():
        ref = KAT[dname][key]
        lims, priors, prargs = getattr(ss, f'set_{b.type_}')(b, **kw)
        np.testing.assert_allclose(np.array(lims, dtype=float), np.array(ref['limits'], dtype=float),
                                   rtol=1e-15, err_msg=f'{dname} {key}')
        assert list(priors) == ref['priors'], (dname, key)
        got = [None if a is None else [float(x) for x in a] for a in prargs]
        assert got == ref['prargs'], (dname, key)
