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
  hill_kat.npz      -- the reference's own Hill prior (support/priors/Hill.prior
                       with math_utils.cps, executed from the reference's
                       files) at seeded planet sets, to pin the oracle's
                       restatement
  gp_kat.npz        -- oracle (logL, logprior) of the celerite GP cases (the
                       recursion, checked against the dense definition when
                       written), to keep the GP oracle stable across machines
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
    hill_fixture(ref_root)
    gp_fixture(arr)


def gp_fixture(arr):
    """Oracle GP log-likelihoods of gp_case_models, each checked against the
    dense-Cholesky definition before it is written."""
    from oracle import gp
    from tests.golden.cases import gp_case_models
    out = {}
    for name, (m, d, th) in gp_case_models(arr).items():
        o = OracleRV(m.spec(), d.as_dict())
        (terms,) = [b['gp_terms'] for b in o.blocks if b['type'] == 'Celerite2']
        lp = np.array([o.my_prior(t) for t in th])
        ll = np.full(len(th), -np.inf)
        for i, t in enumerate(th):
            if not np.isfinite(lp[i]):
                continue
            ll[i] = o.my_likelihood(t)
            model, err2 = o.my_model(t)
            full = o.full_theta(t)
            co = gp.coefficients([(k, [full[j] for j in sl]) for k, sl in terms])
            dense = gp.dense_loglike(o.X_, o.Y_ - model, err2, co)
            assert abs(ll[i] - dense) <= 1e-10 * abs(dense), (name, i)
        out[f'{name}__theta'] = th
        out[f'{name}__logl'] = ll
        out[f'{name}__logprior'] = lp
    np.savez_compressed(os.path.join(HERE, 'gp_kat.npz'), **out)
    print('gp_kat:', sorted(k for k in out if k.endswith('__logl')))


def hill_fixture(ref_root):
    """Evaluate the reference's Hill prior on seeded planet sets."""
    import importlib.util
    src = os.path.join(ref_root, 'src', 'astroemperor')
    spec = importlib.util.spec_from_file_location('_ref_math_utils', os.path.join(src, 'math_utils.py'))
    mu = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mu)
    ns = {'np': np, 'cps': mu.cps}
    exec(open(os.path.join(src, 'support', 'priors', 'Hill.prior')).read(), ns)
    rng = np.random.default_rng(4321)
    X, A, out = [], [], []
    for i in range(400):
        k = int(rng.integers(2, 5))
        per = np.exp(rng.uniform(np.log(2.0), np.log(300.0), k))
        amp = np.exp(rng.uniform(np.log(0.5), np.log(60.0), k))
        ecc = rng.uniform(0.0, 0.4, k)
        mstar = float(rng.uniform(0.3, 1.5))
        x = np.zeros((3, 4))
        x[:, :k] = [per, amp, ecc]
        with np.errstate(all='ignore'):
            v = ns['Hill'](np.array([per, amp, ecc]), [None, None], [k, mstar])
        X.append(x)
        A.append([k, mstar])
        out.append(v)
    np.savez_compressed(os.path.join(HERE, 'hill_kat.npz'), x=np.array(X), args=np.array(A),
                        value=np.array(out))
    print('hill_kat:', int(np.sum(np.isfinite(out))), 'stable of', len(out))


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else '/root/reference')
