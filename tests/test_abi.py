"""The C ABI: exported symbols, struct layouts, host-side validation.

Runs without a GPU: every check here stops before the first CUDA call.
"""
import ctypes as C
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from astroemperor_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'emp_gpu.h')


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r'/\*.*?\*/', '', txt, flags=re.S)
    return sorted(set(re.findall(r'\b(emp_[a-z0-9_]+)\s*\(', txt)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(N.SIGNATURES), set(names) ^ set(N.SIGNATURES)


def test_abi_version(lib):
    assert lib.emp_abi_version() == N.EMP_ABI_VERSION


LAYOUT_C = r'''
#include <stdio.h>
#include <stddef.h>
#include "emp_gpu.h"
#define P(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  printf("emp_prior %zu\nemp_model_desc %zu\nemp_dataset_desc %zu\nemp_pt_state %zu\nemp_pt_record %zu\n"
         "emp_am_desc %zu\n",
         sizeof(emp_prior), sizeof(emp_model_desc), sizeof(emp_dataset_desc),
         sizeof(emp_pt_state), sizeof(emp_pt_record), sizeof(emp_am_desc));
  P(emp_model_desc, am_on) P(emp_model_desc, am_jitter_slot)
  P(emp_am_desc, catalogs) P(emp_am_desc, gsv) P(emp_am_desc, common_t)
  P(emp_model_desc, kep_param) P(emp_model_desc, full_fixed) P(emp_model_desc, prior)
  P(emp_model_desc, prior_slot) P(emp_model_desc, derived) P(emp_model_desc, loglike_const)
  P(emp_pt_state, theta) P(emp_pt_state, n_perm_units) P(emp_pt_state, seed)
  P(emp_pt_state, adapt_mode) P(emp_pt_state, precision)
  P(emp_pt_record, chain) P(emp_pt_record, n_recorded)
  P(emp_dataset_desc, offsets) P(emp_dataset_desc, inst)
  return 0;
}
'''


@pytest.mark.skipif(shutil.which('gcc') is None, reason='gcc not available')
def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / 'layout.c'
    src.write_text(LAYOUT_C)
    exe = tmp_path / 'layout'
    subprocess.run(['gcc', '-I', os.path.join(ROOT, 'include'), str(src), '-o', str(exe)], check=True)
    out = dict(l.rsplit(' ', 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                         check=True).stdout.strip().splitlines())
    types = {'emp_prior': N.EmpPrior, 'emp_model_desc': N.EmpModelDesc,
             'emp_dataset_desc': N.EmpDatasetDesc, 'emp_pt_state': N.EmpPtState,
             'emp_pt_record': N.EmpPtRecord, 'emp_am_desc': N.EmpAmDesc}
    for k, v in out.items():
        if '.' in k:
            t, f = k.split('.')
            assert getattr(types[t], f).offset == int(v), k
        else:
            assert C.sizeof(types[k]) == int(v), k


def _desc_1planet():
    from astroemperor_gb300.data import preprocess_instruments
    from astroemperor_gb300.model import JitterBlock, KeplerianBlock, OffsetBlock, ReddModel, SmartSetter
    rng = np.random.default_rng(3)
    t = np.sort(rng.uniform(0, 100, 40))
    arr = np.column_stack([t + 2450000, rng.normal(0, 5, 40), np.full(40, 2.0)])
    d = preprocess_instruments([arr])
    ss = SmartSetter(d)
    kb = KeplerianBlock(1, 1); ss(kb)
    ob = OffsetBlock(1); ss(ob)
    jb = JitterBlock(1); ss(jb)
    return ReddModel([kb, ob, jb], d), d


def _dataset(t, y, e, ins):
    keep = dict(t=np.ascontiguousarray(t, dtype=np.float64), y=np.ascontiguousarray(y, dtype=np.float64),
                e=np.ascontiguousarray(e, dtype=np.float64), i=np.ascontiguousarray(ins, dtype=np.int32),
                o=np.array([0, len(t)], dtype=np.int64))
    ds = N.EmpDatasetDesc()
    ds.n_systems = 1
    ds.offsets = keep['o'].ctypes.data_as(C.POINTER(C.c_int64))
    ds.t = keep['t'].ctypes.data_as(C.POINTER(C.c_double))
    ds.y = keep['y'].ctypes.data_as(C.POINTER(C.c_double))
    ds.yerr = keep['e'].ctypes.data_as(C.POINTER(C.c_double))
    ds.inst = keep['i'].ctypes.data_as(C.POINTER(C.c_int32))
    return ds, keep


def _create(lib, md, ds):
    h = C.c_void_p()
    rc = lib.emp_create(C.byref(md), C.byref(ds), C.byref(h))
    return rc, lib.emp_last_error_string().decode()


def test_create_rejects_bad_datasets_before_touching_the_gpu(lib):
    m, d = _desc_1planet()
    md = m.descriptor()
    n = d.ndata
    # zero epochs
    ds, keep = _dataset(d.BJD[:0], d.RV[:0], d.eRV[:0], d.Flag[:0])
    rc, msg = _create(lib, md, ds)
    assert rc == N.EMP_E_INVALID and 'epochs' in msg
    # instrument id out of range
    bad = d.Flag.copy(); bad[3] = 2
    ds, keep = _dataset(d.BJD, d.RV, d.eRV, bad)
    assert _create(lib, md, ds)[0] == N.EMP_E_INVALID
    # NaN value
    y = d.RV.copy(); y[5] = np.nan
    ds, keep = _dataset(d.BJD, y, d.eRV, d.Flag)
    rc, msg = _create(lib, md, ds)
    assert rc == N.EMP_E_INVALID and 'non-finite' in msg
    # unsorted times
    t = d.BJD.copy(); t[[1, 2]] = t[[2, 1]]
    ds, keep = _dataset(t, d.RV, d.eRV, d.Flag)
    assert _create(lib, md, ds)[0] == N.EMP_E_INVALID
    # more than one system through the single-system entry
    ds, keep = _dataset(d.BJD, d.RV, d.eRV, d.Flag)
    ds.n_systems = 2
    assert _create(lib, md, ds)[0] == N.EMP_E_UNSUPPORTED


def test_create_rejects_bad_descriptors(lib):
    m, d = _desc_1planet()
    ds, keep = _dataset(d.BJD, d.RV, d.eRV, d.Flag)
    md = m.descriptor(); md.abi_version = 99
    assert _create(lib, md, ds)[0] == N.EMP_E_INVALID
    md = m.descriptor(); md.kep_param[0] = 5
    assert _create(lib, md, ds)[0] == N.EMP_E_UNSUPPORTED
    md = m.descriptor(); md.n_free = md.n_full + 1
    assert _create(lib, md, ds)[0] == N.EMP_E_INVALID
    md = m.descriptor(); md.full_src[0] = 1          # free index 1 mapped twice
    assert _create(lib, md, ds)[0] == N.EMP_E_INVALID
    md = m.descriptor(); md.ma_order = 4
    assert _create(lib, md, ds)[0] == N.EMP_E_SIZE
    md = m.descriptor(); md.prior[0].kind = 9
    assert _create(lib, md, ds)[0] == N.EMP_E_INVALID
    md = m.descriptor(); md.prior[1].a1 = 0.0; md.prior[1].kind = 1
    assert _create(lib, md, ds)[0] == N.EMP_E_INVALID


def test_null_handles_are_errors_not_crashes(lib):
    assert lib.emp_logpost(None, None, 1, None, None, None, None, None, 0, None) == N.EMP_E_INVALID
    assert lib.emp_pt_run(None, None, None, 1, 1, None) == N.EMP_E_INVALID
    assert lib.emp_pt_sweep(None, None, None, None) == N.EMP_E_INVALID
    assert lib.emp_model_eval(None, None, 1, None, None, None) == N.EMP_E_INVALID
    assert lib.emp_set_launch(None, 0, 32, 0) == N.EMP_E_INVALID
    assert lib.emp_destroy(None) == N.EMP_OK
    assert b'NULL' in lib.emp_last_error_string()
    am = N.EmpAmDesc()
    assert lib.emp_set_astrometry(None, C.byref(am)) == N.EMP_E_INVALID
    assert lib.emp_logpost_grad(None, None, 1, None, None, None, None, None) == N.EMP_E_INVALID


def test_history_reductions_reject_bad_arguments(lib):
    # emp_ladder_sums / emp_autocorr check their arguments before any launch
    buf = C.c_void_p(16)            # never dereferenced: the checks fail first
    assert lib.emp_ladder_sums(None, 10, 2, 4, 0, 1, None, None, 0, buf, None, None) == N.EMP_E_INVALID
    assert lib.emp_ladder_sums(buf, 10, 0, 4, 0, 1, None, None, 0, buf, None, None) == N.EMP_E_INVALID
    assert lib.emp_ladder_sums(buf, 10, 2, 4, 0, 0, None, None, 0, buf, None, None) == N.EMP_E_INVALID
    assert lib.emp_ladder_sums(buf, 10, 2, 4, 0, 1, None, None, 3, buf, None, None) == N.EMP_E_INVALID
    assert lib.emp_autocorr(None, 10, 2, 4, 3, 0, 1, 8, buf, None) == N.EMP_E_INVALID
    assert lib.emp_autocorr(buf, 10, 2, 4, 3, 0, 1, 0, buf, None) == N.EMP_E_INVALID
    assert lib.emp_autocorr(buf, 60000, 1, 2, 1, 0, 1, 8, buf, None) == N.EMP_E_SIZE


def _batch(lib, models, parts):
    """emp_create_batch over per-system (t, y, e, ins) tuples."""
    S = len(models)
    descs = (N.EmpModelDesc * S)()
    for s, m in enumerate(models):
        descs[s] = m.descriptor() if hasattr(m, 'descriptor') else m
    cat = lambda k, dt: np.ascontiguousarray(np.concatenate([p[k] for p in parts]), dtype=dt)
    keep = dict(t=cat(0, np.float64), y=cat(1, np.float64), e=cat(2, np.float64), i=cat(3, np.int32),
                o=np.concatenate([[0], np.cumsum([len(p[0]) for p in parts])]).astype(np.int64))
    ds = N.EmpDatasetDesc()
    ds.n_systems = S
    ds.offsets = keep['o'].ctypes.data_as(C.POINTER(C.c_int64))
    ds.t = keep['t'].ctypes.data_as(C.POINTER(C.c_double))
    ds.y = keep['y'].ctypes.data_as(C.POINTER(C.c_double))
    ds.yerr = keep['e'].ctypes.data_as(C.POINTER(C.c_double))
    ds.inst = keep['i'].ctypes.data_as(C.POINTER(C.c_int32))
    h = C.c_void_p()
    rc = lib.emp_create_batch(descs, C.byref(ds), C.byref(h))
    return rc, lib.emp_last_error_string().decode()


def test_create_batch_rejects_bad_input_before_touching_the_gpu(lib):
    from astroemperor_gb300 import synth
    sy = synth.make_ragged(3, seed=1)
    models = [m for m, _, _ in sy]
    parts = [(d.BJD, d.RV, d.eRV, d.Flag) for _, d, _ in sy]
    # a system with no epochs
    bad = list(parts)
    bad[1] = tuple(x[:0] for x in parts[1])
    rc, msg = _batch(lib, models, bad)
    assert rc == N.EMP_E_INVALID and 'system 1' in msg
    # unsorted times in the last system
    t = parts[2][0].copy(); t[[0, 1]] = t[[1, 0]]
    bad = list(parts); bad[2] = (t,) + tuple(parts[2][1:])
    rc, msg = _batch(lib, models, bad)
    assert rc == N.EMP_E_INVALID and 'system 2' in msg and 'sorted' in msg
    # a bad descriptor names its system
    md = models[1].descriptor(); md.abi_version = 99
    rc, msg = _batch(lib, [models[0], md, models[2]], parts)
    assert rc == N.EMP_E_INVALID and 'system 1' in msg
    # MA order must agree across systems
    md = models[2].descriptor(); md.ma_order = 1; md.ma_slot = 0; md.ma_global = 1
    rc, msg = _batch(lib, [models[0], models[1], md], parts)
    assert rc == N.EMP_E_UNSUPPORTED and 'MA order' in msg
    # system count out of range
    descs = (N.EmpModelDesc * 1)()
    ds = N.EmpDatasetDesc(); ds.n_systems = 0
    h = C.c_void_p()
    assert lib.emp_create_batch(descs, C.byref(ds), C.byref(h)) == N.EMP_E_SIZE
    assert lib.emp_num_systems(None) == N.EMP_E_INVALID


def test_create_rejects_bad_gp_and_hill_fields(lib, peg_arr):
    """GP and Hill descriptor fields are checked before any device work."""
    from tests.golden.cases import GP_KERNELS, model_51peg
    m, d = model_51peg(peg_arr, k=1, par=1, gp=GP_KERNELS['grot'])
    ds, keep = _dataset(d.BJD, d.RV, d.eRV, d.Flag)
    md = m.descriptor(); md.gp_kind[0] = 7                    # unknown term kind
    rc, msg = _create(lib, md, ds)
    assert rc == N.EMP_E_UNSUPPORTED and 'kind' in msg
    md = m.descriptor(); md.gp_slot[0][1] = md.n_full         # parameter slot out of range
    rc, msg = _create(lib, md, ds)
    assert rc == N.EMP_E_INVALID and 'slot' in msg
    md = m.descriptor(); md.gp_slot[0][4] = 0                 # unused parameter must be -1
    assert _create(lib, md, ds)[0] == N.EMP_E_INVALID
    md = m.descriptor(); md.gp_nterms = N.EMP_MAX_GP_TERMS + 1
    assert _create(lib, md, ds)[0] == N.EMP_E_SIZE
    md = m.descriptor()                                       # 5 rotation terms: 20 dimensions
    md.gp_nterms = 5
    for j in range(5):
        md.gp_kind[j] = N.EMP_GP_GROT
        for i in range(5):
            md.gp_slot[j][i] = md.gp_slot[0][i]
    rc, msg = _create(lib, md, ds)
    assert rc == N.EMP_E_UNSUPPORTED and 'dimensions' in msg
    # Hill priors
    m2, d2 = model_51peg(peg_arr, k=2, par=1, hill=1.1)
    ds2, keep2 = _dataset(d2.BJD, d2.RV, d2.eRV, d2.Flag)
    md = m2.descriptor(); md.hill_mask = 1 << 3               # over 3 planets, the model has 2
    assert _create(lib, md, ds2)[0] == N.EMP_E_INVALID
    md = m2.descriptor(); md.hill_mask = 1 << 1               # planet counts start at 2
    assert _create(lib, md, ds2)[0] == N.EMP_E_INVALID
    md = m2.descriptor(); md.hill_starmass = 0.0
    assert _create(lib, md, ds2)[0] == N.EMP_E_INVALID
    md = m2.descriptor(); md.kep_param[0] = 7                 # no PAE script for param. 7
    md.kep_param[1] = 7
    rc, msg = _create(lib, md, ds2)
    assert rc == N.EMP_E_UNSUPPORTED and 'Hill' in msg


def test_mixed_astrometry_batch_rejected_before_touching_the_gpu(lib, peg_arr):
    from tests.golden.cases import model_51peg, model_hip21850
    fix = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'hip21850.npz'))
    m, d, _ = model_hip21850(fix)
    m2, d2 = model_51peg(peg_arr, k=1, par=1)
    parts = [(d.BJD, d.RV, d.eRV, d.Flag), (d2.BJD, d2.RV, d2.eRV, d2.Flag)]
    rc, msg = _batch(lib, [m, m2], parts)
    assert rc == N.EMP_E_UNSUPPORTED and 'astrometric and RV-only' in msg
