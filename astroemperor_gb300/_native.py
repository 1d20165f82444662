"""ctypes binding of ``libemp_gpu.so`` (declared in ``include/emp_gpu.h``).

The structures below mirror the C declarations field for field; ctypes
applies the platform C layout rules, so offsets match the header.  Loading
fails loudly: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, '_lib', 'libemp_gpu.so')

EMP_ABI_VERSION = 4
EMP_MAX_PARAMS = 160
EMP_MAX_PLANETS = 16
EMP_MAX_INS = 16
EMP_MAX_MA = 3
EMP_MAX_GP_TERMS = 8

EMP_GP_REAL = 1
EMP_GP_MATERN32 = 2
EMP_GP_ROTATION = 3
EMP_GP_GROT = 4
EMP_GP_SHO = 16

EMP_OK = 0
EMP_E_INVALID = -1
EMP_E_CUDA = -2
EMP_E_UNSUPPORTED = -3
EMP_E_SIZE = -4
EMP_E_STATE = -5

EMP_TERM_SINUSOID = 8
EMP_TERM_CYCLE_1 = 9
EMP_TERM_CYCLE_2 = 10

EMP_PREC_FP64 = 0
EMP_PREC_MIXED = 1
EMP_LAUNCH_GRAD = 2

PRIOR_KIND = {'Uniform': 0, 'Normal': 1, 'Jeffreys': 2, 'Beta': 3, 'None': 4, 'Isotropic': 5}
EMP_PRIOR_NONE = 4


class EmpPrior(C.Structure):
    _fields_ = [('kind', C.c_int32), ('_pad', C.c_int32),
                ('lo', C.c_double), ('hi', C.c_double),
                ('a0', C.c_double), ('a1', C.c_double), ('a2', C.c_double)]


class EmpModelDesc(C.Structure):
    _fields_ = [
        ('abi_version', C.c_int32), ('n_full', C.c_int32), ('n_free', C.c_int32),
        ('n_planets', C.c_int32), ('n_ins', C.c_int32), ('ma_order', C.c_int32),
        ('ma_global', C.c_int32), ('ma_quirk', C.c_int32), ('acc_order', C.c_int32),
        ('offset_slot', C.c_int32), ('jitter_slot', C.c_int32), ('ma_slot', C.c_int32),
        ('acc_slot', C.c_int32), ('_pad0', C.c_int32),
        ('kep_param', C.c_int32 * EMP_MAX_PLANETS),
        ('kep_slot', C.c_int32 * EMP_MAX_PLANETS),
        ('full_src', C.c_int32 * EMP_MAX_PARAMS),
        ('full_fixed', C.c_double * EMP_MAX_PARAMS),
        ('prior', EmpPrior * EMP_MAX_PARAMS),
        ('prior_slot', C.c_int32 * EMP_MAX_PARAMS),
        ('derived', (EmpPrior * 2) * EMP_MAX_PLANETS),
        ('loglike_const', C.c_double),
        ('prior_const', C.c_double),
        ('n_prior_var', C.c_int32), ('_pad1', C.c_int32),
        ('prior_var', C.c_int32 * (EMP_MAX_PARAMS + 2 * EMP_MAX_PLANETS)),
        ('gp_nterms', C.c_int32), ('_pad2', C.c_int32),
        ('gp_kind', C.c_int32 * EMP_MAX_GP_TERMS),
        ('gp_slot', (C.c_int32 * 5) * EMP_MAX_GP_TERMS),
        ('hill_mask', C.c_int32), ('_pad3', C.c_int32), ('hill_starmass', C.c_double),
        ('am_on', C.c_int32), ('am_offset_slot', C.c_int32), ('am_jitter_slot', C.c_int32),
        ('_pad4', C.c_int32),
    ]


class EmpAmDesc(C.Structure):
    _fields_ = [('n_hipp', C.c_int32), ('n_gost', C.c_int32),
                ('catalogs', C.c_void_p), ('inv_cov', C.c_void_p), ('log_det_cov', C.c_void_p),
                ('astro_gost', C.c_void_p), ('hipp', C.c_void_p), ('gost', C.c_void_p),
                ('gsv', C.c_void_p), ('common_t', C.c_double)]


class EmpDatasetDesc(C.Structure):
    _fields_ = [('n_systems', C.c_int32), ('_pad', C.c_int32),
                ('offsets', C.POINTER(C.c_int64)),
                ('t', C.POINTER(C.c_double)), ('y', C.POINTER(C.c_double)),
                ('yerr', C.POINTER(C.c_double)), ('inst', C.POINTER(C.c_int32))]


class EmpPtState(C.Structure):
    _fields_ = [
        ('ntemps', C.c_int32), ('nwalkers', C.c_int32), ('ndim', C.c_int32), ('nsteps', C.c_int32),
        ('theta', C.c_void_p), ('logl', C.c_void_p), ('logprior', C.c_void_p),
        ('members', C.c_void_p), ('betas', C.c_void_p), ('counters', C.c_void_p),
        ('accepted', C.c_void_p), ('swaps_accepted', C.c_void_p), ('perm_units', C.c_void_p),
        ('n_perm_units', C.c_int32), ('adapt', C.c_int32),
        ('seed', C.c_uint64), ('a', C.c_double),
        ('adapt_tau', C.c_double), ('adapt_nu', C.c_double),
        ('adapt_mode', C.c_int32), ('precision', C.c_int32),
        ('work', C.c_void_p), ('work_bytes', C.c_int64),
        ('n_systems', C.c_int32), ('_pad2', C.c_int32),
    ]


class EmpPtRecord(C.Structure):
    _fields_ = [
        ('capacity', C.c_int64), ('thin', C.c_int32), ('_pad', C.c_int32),
        ('chain', C.c_void_p), ('log_like', C.c_void_p), ('log_prob', C.c_void_p),
        ('beta_history', C.c_void_p), ('tsw_history', C.c_void_p), ('smd_history', C.c_void_p),
        ('n_recorded', C.c_void_p),
    ]


# every symbol include/emp_gpu.h declares, with its ctypes signature
SIGNATURES = {
    'emp_create': (C.c_int, [C.POINTER(EmpModelDesc), C.POINTER(EmpDatasetDesc), C.POINTER(C.c_void_p)]),
    'emp_destroy': (C.c_int, [C.c_void_p]),
    'emp_create_batch': (C.c_int, [C.POINTER(EmpModelDesc), C.POINTER(EmpDatasetDesc), C.POINTER(C.c_void_p)]),
    'emp_num_systems': (C.c_int, [C.c_void_p]),
    'emp_logpost': (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    'emp_logpost_grad': (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p]),
    'emp_set_astrometry': (C.c_int, [C.c_void_p, C.POINTER(EmpAmDesc)]),
    'emp_model_eval': (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    'emp_gp_logl': (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_int, C.c_void_p]),
    'emp_pt_sweep': (C.c_int, [C.c_void_p, C.POINTER(EmpPtState), C.POINTER(EmpPtRecord), C.c_void_p]),
    'emp_pt_sweep_static': (C.c_int, [C.c_void_p, C.POINTER(EmpPtState), C.POINTER(EmpPtRecord),
                                      C.c_void_p]),
    'emp_pt_run': (C.c_int, [C.c_void_p, C.POINTER(EmpPtState), C.POINTER(EmpPtRecord), C.c_int,
                             C.c_int, C.c_void_p]),
    'emp_pt_evaluate': (C.c_int, [C.c_void_p, C.POINTER(EmpPtState), C.c_void_p]),
    'emp_pt_run_host': (C.c_int, [C.c_void_p, C.POINTER(EmpPtState), C.POINTER(EmpPtRecord), C.c_void_p,
                                  C.c_void_p]),
    'emp_pt_work_bytes': (C.c_int64, [C.c_int, C.c_int, C.c_int]),
    'emp_set_launch': (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    'emp_get_launch': (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    'emp_ladder_sums': (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                  C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    'emp_autocorr': (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                               C.c_void_p, C.c_void_p]),
    'emp_probe_peaks': (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p]),
    'emp_launch_count': (C.c_int64, []),
    'emp_last_error_string': (C.c_char_p, []),
    'emp_abi_version': (C.c_int, []),
}


class EmpError(RuntimeError):
    """A non-zero status returned by the native library."""

    def __init__(self, code, func, msg):
        super().__init__(f'{func} returned {code}: {msg}')
        self.code = code


_LIB = None


def load(path: str = LIB_PATH):
    """Load the library (once) and declare every signature; raises if absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise ImportError(
            f'{path} is missing: build it with astroemperor_gb300.build.build() '
            '(there is no CPU fallback for the EMPEROR GPU engine)')
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.emp_abi_version() != EMP_ABI_VERSION:
        raise ImportError(f'libemp_gpu ABI {lib.emp_abi_version()} != {EMP_ABI_VERSION}')
    _LIB = lib
    return lib


def check(rc: int, func: str):
    if rc != EMP_OK:
        msg = load().emp_last_error_string()
        raise EmpError(rc, func, msg.decode() if msg else '')
    return rc


def call(name: str, *args):
    lib = load()
    return check(getattr(lib, name)(*args), name)
