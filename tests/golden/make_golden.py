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
  template_kat.npz  -- my_model / my_likelihood of the known-answer model cases
                       evaluated by the reference's own model templates
                       (support/models/*.model, support/likelihoods/00.like),
                       assembled in the order of emp_model.py:706-781, and its
                       prior templates (support/priors/*.prior) at seeded
                       points; the Kepler equation (kepler.py, absent) is
                       solved by the oracle's solver, so these pin everything
                       else of the oracle's model, likelihood and priors.
                       The documented per-instrument MA (which the reference's
                       own per-instrument template does not compute) is pinned
                       to its live global template moav01.model run on each
                       instrument's time-ordered subsequence
  gj876_rv.npz      -- the reference's tests/datafiles/GJ876/RV/*.vels (eight
                       instruments; BJD, RV, eRV columns of each, the files in
                       the sorted order the reference reads them)
  hip21850.npz      -- the reference's HIP 21850 RV and astrometric data and the
                       Gaia dead-time tables of its support folder, as arrays
  am_kat.npz        -- loglike_AM of the HIP 21850 model (and, keys k2__*, of a
                       two-planet variant) at seeded theta by the
                       reference's own generated astrometry functions
                       (ReddModel._write_model_AM text with constants.scr), and
                       the oracle's (logL, logprior) of the a00.like model, with
                       logL also with the astrometric propagation in long double
  smartsetter_kat.json -- default limits / priors / prargs of every block type
                       as the reference's SmartSetter methods (block_repo.py,
                       run from its source on a small column shim) set them
                       for the 51 Peg data and the two-instrument C2 data
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.rv import OracleRV, preprocess  # noqa: E402
from tests.golden.cases import kat_cases, peg_data  # noqa: E402


def main(ref_root):
    vels = os.path.join(ref_root, 'tests', 'datafiles', '51Peg', 'RV', '51peg.vels')
    arr = np.loadtxt(vels)
    np.savez_compressed(os.path.join(HERE, '51peg_rv.npz'), data=arr)
    gj876_fixture(ref_root)
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
    template_fixture(ref_root, arr)
    smartsetter_fixture(ref_root, arr)
    hip21850_fixture(ref_root)
    am_fixture(ref_root)


def gj876_fixture(ref_root):
    """The GJ 876 RV files as the reference's DataWrapper lists them (sorted)."""
    folder = os.path.join(ref_root, 'tests', 'datafiles', 'GJ876', 'RV')
    names = [fn for fn in sorted(os.listdir(folder)) if fn != '.DS_Store']
    out = {'names': np.array(names)}
    for k, fn in enumerate(names):
        out[f'ins_{k}'] = np.loadtxt(os.path.join(folder, fn), ndmin=2)[:, :3]
    np.savez_compressed(os.path.join(HERE, 'gj876_rv.npz'), **out)
    print('gj876_rv:', names)


class _Col:
    """The few pandas Series operations SmartSetter uses."""

    def __init__(self, v):
        self.v = np.asarray(v, dtype=float)

    def std(self, ddof=1):
        return float(np.std(self.v, ddof=ddof))

    def max(self):
        return float(np.max(self.v))

    def min(self):
        return float(np.min(self.v))

    def abs(self):
        return _Col(np.abs(self.v))

    def __eq__(self, other):
        return self.v == other


class _Frame:
    def __init__(self, cols):
        self.cols = {k: np.asarray(v) for k, v in cols.items()}

    def __getitem__(self, key):
        if isinstance(key, str):
            return _Col(self.cols[key])
        return _Frame({c: v[key] for c, v in self.cols.items()})


def smartsetter_fixture(ref_root, arr):
    """The reference's SmartSetter limit methods run from block_repo.py's source."""
    import ast
    import json
    import types
    from astroemperor_gb300 import synth
    text = open(os.path.join(ref_root, 'src', 'astroemperor', 'block_repo.py')).read()
    tree = ast.parse(text)
    cls = next(n for n in ast.walk(tree) if isinstance(n, ast.ClassDef) and n.name == 'SmartSetter')
    names = ['__init__', 'set_Keplerian', 'set_Offset', 'set_Jitter', 'set_MOAV', 'set_Acceleration',
             'set_Sinusoid', 'set_MagneticCycle']
    parts = [ast.get_source_segment(text, n) for n in cls.body
             if isinstance(n, ast.FunctionDef) and n.name in names]
    src = 'class RefSmartSetter(object):\n' + '\n'.join('    ' + l for p in parts for l in p.split('\n'))
    g = {'np': np}
    exec(src, g)
    Ref = g['RefSmartSetter']
    # the additional-parameter helpers only attach derived parameters
    Ref.ecc_w_add_additional = lambda self, b, **kw: None
    Ref.per_add_additional = lambda self, b, **kw: None

    def clean(x):
        if isinstance(x, (list, tuple)):
            return [clean(v) for v in x]
        if x is None:
            return None
        return float(x)

    out = {}
    _, d2, _, _ = synth.build_model('c2', seed=1234)
    for dname, d in (('51peg', peg_data(arr)), ('c2', d2)):
        ref = Ref(_Frame({'BJD': d.BJD, 'RV': d.RV, 'eRV': d.eRV, 'Flag': d.Flag}))
        res = {}
        for par in (0, 1, 2, 3, 4, 6, 7):
            b = types.SimpleNamespace(parameterisation=par, astrometry_bool=False, number_=1)
            res[f'Keplerian{par}'] = ref.set_Keplerian(b, prargs=[[0, 1], [0, 0.1]], starmass=None,
                                                       dynamics=False, kplan=1, dynamics_already_included=False)
        nins = d.nins
        res['Offset'] = ref.set_Offset(types.SimpleNamespace(number_=nins))
        res['Jitter'] = ref.set_Jitter(types.SimpleNamespace(number_=nins), [0, 1], [5, 5])
        res['MOAV2'] = ref.set_MOAV(types.SimpleNamespace(number_=nins, moav=2))
        res['Acceleration2'] = ref.set_Acceleration(types.SimpleNamespace(number_=2))
        res['Sinusoid'] = ref.set_Sinusoid(types.SimpleNamespace(number_=1))
        res['MagneticCycle'] = ref.set_MagneticCycle(types.SimpleNamespace(number_=1))
        out[dname] = {k: {'limits': clean(v[0]), 'priors': list(v[1]), 'prargs': clean(v[2])}
                      for k, v in res.items()}
    with open(os.path.join(HERE, 'smartsetter_kat.json'), 'w') as f:
        json.dump(out, f, indent=1)
    print('smartsetter_kat:', {k: len(v) for k, v in out.items()})


def _template_model_source(model, support):
    """The reference's my_model text for a model of this package's layer:
    each block's template formatted with the block's write_args (block_repo.py),
    in the assembly order of emp_model.py:706-781."""
    def tpl(name):
        return open(os.path.join(support, 'models', name)).read()
    nins = model.data.nins
    helpers = []
    src = ['def my_model(theta):',
           '    for a in A_:',
           '        theta = np.insert(theta, a, mod_fixed_[a])',
           '    model0 = np.zeros(ndat)',
           '    err20 = YERR_ ** 2']
    for b in model.blocks:
        sl = b.slice
        if b.type_ == 'Keplerian':
            src.append(tpl(f'kep0{b.parameterisation}.model').format(sl))
        elif b.type_ == 'Offset':
            for k in range(1, nins + 1):
                src.append(tpl('offset00.model').format(k, sl))
        elif b.type_ in ('Sinusoid', 'MagneticCycle', 'Acceleration'):
            name = {'Sinusoid': 'sinusoid00.model', 'MagneticCycle': 'magneticcycle00.model',
                    'Acceleration': 'acc.model'}[b.type_]
            src.append(tpl(name).format(sl))
        elif b.type_ == 'MOAV':
            src.append('    residuals = Y_ - model0')
            if b.is_global:
                src.append(tpl('moav01.model').format(nins, sl, b.moav))
            elif model.moav_reference_quirk:
                for k in range(1, nins + 1):
                    src.append(tpl('moav00.model').format(k, sl, b.moav))
            else:
                # the documented per-instrument MA (docs/user-guide/ug-the-model.md):
                # the reference's live template moav01 run on each instrument's
                # time-ordered subsequence with that instrument's coefficients
                for k in range(1, nins + 1):
                    q0 = sl.start + 2 * b.moav * (k - 1)
                    body = tpl('moav01.model').format(nins, f'{q0}:{q0 + 2 * b.moav}', b.moav)
                    helpers.append(f'def _ma_run{k}(theta, X_, residuals, model0, ndat):\n{body}\n'
                                   '    return model0, residuals\n')
                    src.append(f'    model0[mask{k}], residuals[mask{k}] = _ma_run{k}('
                               f'theta, X_[mask{k}], residuals[mask{k}].copy(), model0[mask{k}].copy(), '
                               f'ndat{k})')
        elif b.type_ == 'Jitter':
            for k in range(1, nins + 1):
                src.append(tpl('jitter00.model').format(k, sl))
        else:
            raise ValueError(b.type_)
    src.append('    return model0, err20')
    return ''.join(helpers) + '\n'.join(src) + '\n'


def _reference_check_prargs(src_dir):
    """The reference's prargs normaliser (emp_model.py, Parameter_Block
    _check_prargs / _check_additional_prargs), taken from its source and run
    on duck-typed parameters: returns f(params) normalising in place."""
    import ast
    from scipy.stats import norm
    text = open(os.path.join(src_dir, 'emp_model.py')).read()
    tree = ast.parse(text)
    fn = None
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == '_check_prargs':
            fn = node
            break
    code = ast.get_source_segment(text, fn)
    lines = code.split('\n')
    indent = len(lines[0]) - len(lines[0].lstrip())
    code = '\n'.join(l[indent:] for l in lines)
    g = {'np': np, 'norm': norm}
    exec(code, g)
    return lambda params: g['_check_prargs'](list(params))


def _template_prior_source(model, src_dir, normalise):
    """The reference's my_prior text (emp.py:182-254) for a model of this
    package's layer: one prior call per free parameter with the normalised
    prargs, the block's -inf exit, then the derived priors (Amp, Ecc, Hill)."""
    import copy
    support = os.path.join(src_dir, 'support')
    C_ = list(model.C_)
    out = ['def my_prior(theta):', '    for a in A_:', '        theta = np.insert(theta, a, mod_fixed_[a])',
           '    lp = 0.']
    count = 0
    for b in model.blocks:
        free = [copy.copy(p) for p in b if p.fixed is None]
        normalise(free)
        for p in free:
            out.append(f'    lp += {p.prior}(theta[{C_[count]}], {p.limits}, {p.prargs})')
            count += 1
        out.append('    if lp == -np.inf:\n        return lp')
        extra = [copy.copy(p) for p in getattr(b, 'additional_parameters', []) if getattr(p, 'has_prior', False)]
        normalise(extra)
        for p in extra:
            if p.name[:3] == 'Amp':
                out.append(f'    x = theta[{b.slice}][1]**2 + theta[{b.slice}][2]**2')
            elif p.name[:3] == 'Ecc':
                out.append(f'    x = theta[{b.slice}][3]**2 + theta[{b.slice}][4]**2')
            elif p.name == 'Hill' and p.prargs[0] > 1:
                out.append(f'    b_len = {len(b)}\n    kplanets = {p.prargs[0]}')
                out.append(open(os.path.join(support, 'PAE', f'0{b.parameterisation}.pae')).read())
            else:
                continue
            out.append(f'    lp += {p.prior}(x, {p.limits}, {p.prargs})')
    out.append('    return lp')
    return '\n'.join(out) + '\n'


def template_fixture(ref_root, arr):
    """The reference's own templates on the known-answer cases (see module doc)."""
    import types
    from oracle.rv import kepler_solve, PRIORS, check_prargs
    from tests.golden.cases import kat_case_models
    import importlib.util
    from scipy.stats import beta as betapdf          # the reference's model dependency (emp.py:428)
    src_dir = os.path.join(ref_root, 'src', 'astroemperor')
    support = os.path.join(src_dir, 'support')
    like_src = open(os.path.join(support, 'likelihoods', '00.like')).read()
    normalise = _reference_check_prargs(src_dir)
    spec = importlib.util.spec_from_file_location('_ref_math_utils', os.path.join(src_dir, 'math_utils.py'))
    mu = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mu)
    prior_defs = ''.join(open(os.path.join(support, 'priors', f)).read() + '\n'
                         for f in sorted(os.listdir(os.path.join(support, 'priors'))))
    out = {}
    for name, (m, d, th) in kat_case_models(arr).items():
        g = {'np': np, 'kepler': types.SimpleNamespace(solve=kepler_solve),
             'X_': d.BJD, 'Y_': d.RV, 'YERR_': d.eRV, 'ndat': d.ndata,
             'A_': list(m.A_), 'mod_fixed_': m.mod_fixed}
        for k in range(1, d.nins + 1):
            g[f'mask{k}'] = d.Flag == k
            g[f'ndat{k}'] = int(np.sum(d.Flag == k))
        exec(_template_model_source(m, support), g)
        exec(like_src, g)
        g.update({'betapdf': betapdf, 'cps': mu.cps})
        exec(prior_defs, g)
        exec(_template_prior_source(m, src_dir, normalise), g)
        # the per-epoch model of the large cases is pinned through logL only
        pick = np.linspace(0, len(th) - 1, 6).astype(int) if d.ndata <= 4096 else np.zeros(0, int)
        mod, err, ll = [], [], []
        with np.errstate(all='ignore'):
            for i, t in enumerate(th):
                a, b = g['my_model'](t)
                if i in pick:
                    mod.append(a)
                    err.append(b)
                ll.append(g['my_likelihood'](t))
        out[f'{name}__pick'] = pick
        out[f'{name}__model'] = np.array(mod)
        out[f'{name}__err2'] = np.array(err)
        out[f'{name}__logl'] = np.array(ll)
        with np.errstate(all='ignore'):
            out[f'{name}__logprior'] = np.array([g['my_prior'](t) for t in th], dtype=np.float64)
    # prior templates at seeded points
    rng = np.random.default_rng(99)
    for prior in ('Uniform', 'Normal', 'Jeffreys', 'Beta'):
        from scipy.stats import beta as betapdf          # the reference's model dependency (emp.py:428)
        gp_ = {'np': np, 'betapdf': betapdf}
        exec(open(os.path.join(support, 'priors', f'{prior}.prior')).read(), gp_)
        fn = gp_[prior]
        xs, vals = [], []
        for _ in range(200):
            lo = rng.uniform(0.01, 1.0)
            hi = lo + rng.uniform(0.1, 3.0)
            lim = [lo, hi] if prior != 'Beta' else [0.0, 1.0]
            x = rng.uniform(lim[0] - 0.2, lim[1] + 0.2)
            pr = {'Normal': [rng.uniform(lo, hi), rng.uniform(0.1, 1.0)], 'Beta': [rng.uniform(0.5, 3.0),
                  rng.uniform(0.5, 3.0)]}.get(prior)
            args = check_prargs(prior, lim, pr)
            with np.errstate(all='ignore'):
                v = fn(x, lim, args)
            xs.append([x, lim[0], lim[1]] + (list(pr) if pr else [np.nan, np.nan]))
            vals.append(v)
        out[f'prior_{prior}__in'] = np.array(xs)
        out[f'prior_{prior}__value'] = np.array(vals, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, 'template_kat.npz'), **out)
    print('template_kat:', sorted(k for k in out if k.endswith('__logl')))


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


def hip21850_fixture(ref_root):
    """The reference's HIP 21850 data (tests/datafiles/HIP21850: four RV files,
    the Hipparcos/Gaia catalogue rows, the Hipparcos abscissae and the Gaia
    scan epochs) and its Gaia dead-time tables (support/deadtime), as
    arrays: tests/golden/hip21850.npz."""
    from astroemperor_gb300.astrometry import _read_csv, _read_whitespace_table, read_deadtime
    base = os.path.join(ref_root, 'tests', 'datafiles', 'HIP21850')
    out = {}
    names = sorted(fn for fn in os.listdir(os.path.join(base, 'RV')) if fn != '.DS_Store')
    out['rv_names'] = np.array(names)
    for k, fn in enumerate(names):
        out[f'rv_{k}'] = np.loadtxt(os.path.join(base, 'RV', fn), ndmin=2)[:, :3]
    am = os.path.join(base, 'AM')
    hg = _read_whitespace_table(os.path.join(am, 'HIP21850_hipgaia.hg123'))
    for k, v in hg.items():
        if v.dtype.kind == 'f':
            out[f'hg_{k}'] = v
    hipp = _read_whitespace_table(os.path.join(am, 'HIP21850_hip2.abs'))
    for k in ('BJD', 'EPOCH', 'PARF', 'CPSI', 'SPSI', 'RES', 'SRES'):
        out[f'hipp_{k}'] = hipp[k]
    g = _read_csv(os.path.join(am, 'HIP21850_gost.csv'))
    out['gost_bjd'] = g['ObservationTimeAtBarycentre[BarycentricJulianDateInTCB]']
    out['gost_psi'] = g['scanAngle[rad]']
    out['gost_parf'] = g['parallaxFactorAlongScan']
    dead = os.path.join(ref_root, 'src', 'astroemperor', 'support', 'deadtime')
    out['dead_dr2'] = read_deadtime(os.path.join(dead, 'astrometric_gaps_gaiadr2_08252020.csv'))
    out['dead_dr3'] = read_deadtime(os.path.join(dead, 'astrometric_gaps_gaiaedr3_12232020.csv'))
    np.savez_compressed(os.path.join(HERE, 'hip21850.npz'), **out)
    print('hip21850:', {k: np.shape(v) for k, v in out.items() if not k.startswith('hg_')})


def _reference_am_text(src_dir, model):
    """The text ReddModel._write_model_AM (emp_model.py:1232-1675) writes for
    this model's blocks, produced by the reference's own method."""
    import ast
    import io
    import textwrap
    import types
    text = open(os.path.join(src_dir, 'emp_model.py')).read()
    tree = ast.parse(text)
    fn = next(n for n in ast.walk(tree) if isinstance(n, ast.FunctionDef) and n.name == '_write_model_AM')
    ns = {'np': np}
    exec(textwrap.dedent(ast.get_source_segment(text, fn)), ns)

    class Fake:
        data_AM = {'AM_cata': True}

        def __iter__(self):
            return iter(types.SimpleNamespace(type_=b.type_, slice=b.slice) for b in model.blocks)
    buf = io.StringIO()
    ns['_write_model_AM'](Fake(), buf)
    return buf.getvalue()


def am_fixture(ref_root):
    """loglike_AM of the HIP 21850 model at seeded theta, evaluated by the
    reference's own generated functions (the text of _write_model_AM with
    support/astrometry/constants.scr) on the data arrays of this package's
    loader; kepler.solve (absent) is the oracle's solver.  Written with the
    oracle's (logL, logprior) of the whole a00.like model:
    tests/golden/am_kat.npz (the two-planet variant under keys k2__*)."""
    from tests.golden.cases import model_hip21850
    fix = np.load(os.path.join(HERE, 'hip21850.npz'))
    out = {}
    for k, pre in ((1, ''), (2, 'k2__')):
        model, data, am = model_hip21850(fix, k)
        out.update(_am_case(ref_root, model, data, am, pre))
    np.savez_compressed(os.path.join(HERE, 'am_kat.npz'), **out)
    print('am_kat:', {k: v.shape for k, v in out.items()})


def _am_case(ref_root, model, data, am, pre):
    import types
    from oracle.rv import kepler_solve
    from tests.golden.cases import am_case_thetas
    src_dir = os.path.join(ref_root, 'src', 'astroemperor')
    g = {'np': np, 'kepler': types.SimpleNamespace(solve=kepler_solve)}
    exec(open(os.path.join(src_dir, 'support', 'astrometry', 'constants.scr')).read(), g)
    cat = am.catalogs
    nh, ng = am.n_hipp, am.n_gost
    g.update({
        'AM_catalogs_': cat, 'AM_iref_': -1, 'AM_ref_epoch_': cat[-1, 0],
        'AM_catalogs_times_refed': cat[:, 0] - cat[-1, 0], 'AM_catalogs_obs_ref': cat[-1, 1:],
        'AM_PLX_ref': cat[-1, 3],
        'time_iad_all': np.concatenate([am.hipp['BJD'], am.gost['BJD']]),
        'time_iad_gost_refed': am.gost['BJD'] - cat[-1, 0], 'common_t': am.common_t,
        'N_HIPP': nh, 'N_GOST': ng, 'N_IAD': nh + ng,
        'CPSI_HIPP_': am.hipp['CPSI'], 'SPSI_HIPP_': am.hipp['SPSI'], 'EPOCH_HIPP_': am.hipp['EPOCH'],
        'PARF_HIPP_': am.hipp['PARF'], 'RES_HIPP_': am.hipp['RES'], 'SRES_HIPP_': am.hipp['SRES'],
        'CPSI_GOST_': am.gost['CPSI'], 'SPSI_GOST_': am.gost['SPSI'], 'PARF_GOST_': am.gost['parf'],
        'GAIA_CATS': dict(GDR2=dict(mask=am.masks['GDR2'], row=0, cov_idx=1),
                          GDR3=dict(mask=am.masks['GDR3'], row=1, cov_idx=2)),
        'AM_GSV': am.gsv, 'AM_astro_gost': types.SimpleNamespace(values=am.astro_gost),
        'AM_inv_COV': am.inv_cov, 'AM_log_det_COV': am.log_det_cov,
    })
    exec(_reference_am_text(src_dir, model), g)
    th = am_case_thetas(model)
    from oracle.rv import OracleRV
    o = OracleRV(model.spec(), dict(data.as_dict(), am=am.as_dict()))
    full = [o.full_theta(t) for t in th]
    ref_am = np.array([float(g['loglike_AM'](f)) for f in full])
    lp = np.array([o.my_prior(t) for t in th])
    ll = np.array([o.my_likelihood(t) if np.isfinite(p) else -np.inf for t, p in zip(th, lp)])
    o.am_dtype = np.longdouble
    ll_ld = np.array([o.my_likelihood(t) if np.isfinite(p) else -np.inf for t, p in zip(th, lp)])
    print(f'am_kat {pre or "k1"}:', len(th), 'points;', int(np.isfinite(lp).sum()), 'inside the prior')
    return {pre + 'theta': th, pre + 'loglike_am_ref': ref_am, pre + 'logl': ll, pre + 'logl_ld': ll_ld,
            pre + 'logprior': lp}


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden.py <root of the astroemperor source tree>')
    main(sys.argv[1])
