"""ctypes binding of libyaffgb.so (the C ABI in include/yaffgb.h).

There is no CPU fallback: if the CUDA library cannot be loaded, or no CUDA
device is present, every entry point raises.
"""
import ctypes
import os

import numpy as np

from . import build as _build

YG_OK = 0
YG_ERR_ARG = 1
YG_ERR_CUDA = 2
YG_ERR_NAN = 3
YG_ERR_UNSUPPORTED = 4
YG_ERR_CAPACITY = 5
YG_ERR_DENSITY = 6
YG_ERR_STATE = 7

FP64 = 0
MIXED = 1
MIXED_KAHAN = 2
PRECISIONS = {'fp64': FP64, 'mixed': MIXED, 'mixed_kahan': MIXED_KAHAN}

POT_LJ, POT_MM3, POT_EI = 0, 1, 2
POT_MM3CAP, POT_GRIMME = 3, 4
POT_EXPREP, POT_QMDFFREP, POT_LJCROSS, POT_DAMPDISP, POT_DISP68BJ = 5, 6, 7, 8, 9
TR_NONE, TR_HAMMER, TR_SWITCH3 = 0, 1, 2

PART_PAIR0 = 0
PART_EWALD_RECI = 3
PART_EWALD_CORR = 4
PART_VALENCE = 5
NPART = 6

# same layout as the reference's neigh_row_type (yaff/pes/nlist.h:30-35)
neigh_dtype = np.dtype([('a', 'i8'), ('b', 'i8'), ('d', 'f8'), ('dx', 'f8'), ('dy', 'f8'),
                        ('dz', 'f8'), ('r0', 'i8'), ('r1', 'i8'), ('r2', 'i8')])

# every symbol include/yaffgb.h declares, with its ctypes signature
_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double
SIGNATURES = {
    'yg_status_string': (ctypes.c_char_p, [_I]),
    'yg_last_error': (ctypes.c_char_p, []),
    'yg_create': (_I, [_I64, _I, _P, ctypes.POINTER(_P)]),
    'yg_destroy': (_I, [_P]),
    'yg_set_precision': (_I, [_P, _I]),
    'yg_set_cell': (_I, [_P, _P, _P, _I, _D]),
    'yg_set_positions': (_I, [_P, _P, _I]),
    'yg_set_charges': (_I, [_P, _P]),
    'yg_set_scalings': (_I, [_P, _P, _P, _P, _P, _I64]),
    'yg_set_pair_pot': (_I, [_P, _I, _I, _P, _P, _P, _P, _D, _D, _D, _I, _D]),
    'yg_set_pair_table': (_I, [_P, _I, _I, _I64, _P, _P, _P, _P, _I64, _P, _D, _I, _D]),
    'yg_clear_pair_pots': (_I, [_P]),
    'yg_nlist_build': (_I, [_P, _D, _P, _I64, _I64, ctypes.POINTER(_I64)]),
    'yg_nlist_stats': (_I, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    'yg_nlist_set_capacity': (_I, [_P, _I64]),
    'yg_ewald_info': (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I64)]),
    'yg_ewald_wait': (_I, [_P]),
    'yg_ewald_force_path': (_I, [_P, _I]),
    'yg_ewald_sfac_path': (_I, [_P, _I]),
    'yg_check_wait_timeout': (_I, [_P, _I64, ctypes.POINTER(_I)]),
    'yg_nlist_recompute': (_I, [_P]),
    'yg_nlist_build_async': (_I, [_P, ctypes.c_double, _P, _I64, _I64]),
    'yg_nlist_build_wait': (_I, [_P, ctypes.POINTER(_I64)]),
    'yg_nlist_max_disp2': (_I, [_P, ctypes.POINTER(_D)]),
    'yg_nlist_export': (_I, [_P, _P, _I64, ctypes.POINTER(_I64)]),
    'yg_pair_compute': (_I, [_P, _I, _I]),
    'yg_ewald_setup': (_I, [_P, _D, _D, _P, _D, _I64, _I64]),
    'yg_ewald_reci': (_I, [_P, _I]),
    'yg_ewald_corr': (_I, [_P, _I]),
    'yg_set_valence': (_I, [_P, _P, _I64, _P, _I64, _P, _P, _P, _I64]),
    'yg_valence_compute': (_I, [_P, _I]),
    'yg_get_part': (_I, [_P, _I, _P, _P, _P]),
    'yg_get_total': (_I, [_P, _I, _P, _P, _P, _P]),
    'yg_get_total_add': (_I, [_P, _I, _P, _P, _P, _P]),
    'yg_sync': (_I, [_P]),
    'yg_launch_count': (_I64, [_P]),
    'yg_mem_usage': (_I, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    'yg_pool_usage': (_I, [ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    'yg_md_setup': (_I, [_P, _P, _P, _D, _I, _D, _I64]),
    'yg_md_run': (_I, [_P, _I64, _I, _D, ctypes.POINTER(_I64)]),
    'yg_md_get': (_I, [_P, _P, _P, _P, ctypes.POINTER(_I64)]),
    'yg_md_thermostat': (_I, [_P, _I, _D, _D, _I64, _I, _P, _P, _P, ctypes.c_ulonglong]),
    'yg_md_thermo_get': (_I, [_P, _P, _P, _P]),
    'yg_ewald_prefactors': (_I, [_P, _D, _D, _P, _D, _P]),
    'yg_ewald_structurefactors': (_I, [_P, _I64, _P, _P, _P, _D, _P, _D, _P, _P, _P]),
    'yg_ewald_deltae': (_I, [_P, _P, _P, _P, _P, _I64, _P]),
    'yg_mc_create': (_I, [_P, _P, _D, _P, _D, _D, _D, _P, _D, _D, _I64, _P, _P, _P, _P, _I64, _P, _P, _P, _I64,
                          _I64, _I, _P, ctypes.POINTER(_P)]),
    'yg_mc_destroy': (_I, [_P]),
    'yg_mc_set_precision': (_I, [_P, _I]),
    'yg_mc_set_chain': (_I, [_P, _I64, _I64, _P]),
    'yg_mc_get_chain': (_I, [_P, _I64, ctypes.POINTER(_I64), _P, _P, _P]),
    'yg_mc_prefactors': (_I, [_P, _P, ctypes.POINTER(_I64)]),
    'yg_mc_trials': (_I, [_P, _I64, _P, _P, _P, _P, _P]),
    'yg_mc_apply': (_I, [_P, _I64, _P]),
    'yg_mc_launch_count': (_I64, [_P]),
    'yg_fleet_create': (_I, [_I64, _I, _I64, _I, _I, _P, ctypes.POINTER(_P)]),
    'yg_fleet_destroy': (_I, [_P]),
    'yg_fleet_add': (_I, [_P, _I64, _P, _P, _P, _P, _P, _P, _P, _D, _D, _D, _D, _D, _I64, ctypes.POINTER(_I)]),
    'yg_fleet_remove': (_I, [_P, _I]),
    'yg_fleet_step': (_I, [_P, _I64]),
    'yg_fleet_poll': (_I, [_P, _P, _P]),
    'yg_fleet_get': (_I, [_P, _I, _P, _P, _P, ctypes.POINTER(_I64)]),
    'yg_fleet_usage': (_I, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I), ctypes.POINTER(_I64)]),
    'yg_fleet_launch_count': (_I64, [_P]),
    'yg_ewald_corr_noalloc':(_I, [_P, _P, _I64, _P, _P, _P, _I64, _P, _P, _D, _D, _D, _I64, _I64, _P, _P, _P,
                                   _P]),
}

_lib = None


class YaffGBError(RuntimeError):
    def __init__(self, status, where, detail):
        self.status = status
        RuntimeError.__init__(self, '%s failed: %s (%s)' % (where, detail, status))


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Loads libyaffgb.so (building it first when absent) and binds SIGNATURES."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError('libyaffgb.so not built: run python -m yaff_gb300.build')
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, where):
    if status == YG_OK:
        return
    lib = load()
    detail = lib.yg_last_error().decode(errors='replace')
    if not detail:
        detail = lib.yg_status_string(status).decode()
    if status == YG_ERR_NAN:
        raise ValueError('%s: not-a-number (nan) in the result (%s)' % (where, detail))
    if status == YG_ERR_DENSITY:
        raise ValueError('Atom density too high')
    if status == YG_ERR_ARG:
        raise ValueError('%s: %s' % (where, detail))
    raise YaffGBError(status, where, detail)


def ptr(a):
    """Data pointer of a C-contiguous numpy array (None passes NULL)."""
    if a is None:
        return None
    assert a.flags['C_CONTIGUOUS'], 'array must be C contiguous'
    return a.ctypes.data


def require_cuda():
    """Raises unless a CUDA device is visible to the runtime."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError('yaff_gb300 needs a CUDA device (no CPU fallback exists)')
    torch.cuda.init()
