"""Generate the committed golden fixtures under tests/golden/.

Run from the repository root, in an environment where the reference is
mounted (it reads the reference's own data fixture):

    python tests/golden/make_golden.py /path/to/astroemperor

Writes
  51peg_rv.npz      -- the reference's tests/datafiles/51Peg/RV/51peg.vels
                       (BJD, RV, eRV columns, as loaded by np.loadtxt)
  logpost_kat.npz   -- oracle known-answer vectors: (logL, logprior) of a
                       fixed set of theta for several model specs, used to
                       pin the oracle (CPU tests) and the CUDA path (GPU tests)
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.rv import OracleRV, preprocess  # noqa: E402
from tests.golden.cases import kat_cases  # noqa: E402


def main(ref_root):
    vels = os.path.join(ref_root, 'tests', 'datafiles', '51Peg', 'RV', '51peg.vels')
    arr = np.loadtxt(vels)
    np.savez_compressed(os.path.join(HERE, '51peg_rv.npz'), data=arr)
    out = {}
    specs = {}
    for name, (spec, data, thetas) in kat_cases(arr).items():
        o = OracleRV(spec, data)
        ll = np.array([o.my_likelihood(t) if np.isfinite(o.my_prior(t)) else -np.inf for t in thetas])
        lp = np.array([o.my_prior(t) for t in thetas])
        out[f'{name}__theta'] = thetas
        out[f'{name}__logl'] = ll
        out[f'{name}__logprior'] = lp
        specs[name] = spec
    out['specs_json'] = np.array(json.dumps(specs))
    np.savez_compressed(os.path.join(HERE, 'logpost_kat.npz'), **out)
    print('wrote', sorted(k for k in out if k.endswith('__logl')))


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else '/root/reference')
