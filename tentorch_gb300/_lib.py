'''
The ctypes binding of `libtentorch_gb300.so` (declared in include/tentorch_gb300.h).

The library is built in-tree by `tentorch_gb300.build`; importing this module loads it and fails
loudly when it is missing, because the package has no CPU path for the contraction engine.  Status
codes become the exceptions the reference raises for the same conditions: TT_EINVAL ValueError,
TT_ERANGE IndexError, TT_ELOGIC and TT_ECUDA RuntimeError.
'''
import ctypes
import os

from tentorch_gb300.build import LIBRARY

if not os.path.exists(LIBRARY):
    raise ImportError(f'the engine library {LIBRARY} is not built: run `python tentorch_gb300/build.py`')

lib = ctypes.CDLL(LIBRARY)

i32, i64, f64, vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p
P = ctypes.POINTER


def _declare(name, *args):
    fn = getattr(lib, name)
    fn.argtypes = list(args)
    fn.restype = i32
    return fn


lib.tt_last_error.restype = ctypes.c_char_p
lib.tt_last_error.argtypes = []
lib.tt_version.restype = i32

_declare('tt_category', i32, i64, P(i32))
_declare('tt_outcomes', i32, i64, i64, i32, P(i64), P(i32), P(i32))
_declare('tt_dual', i32, i64, P(i64))
_declare('tt_q_dim', i32, i64, P(f64))
_declare('tt_F_symbol', i32, i64, i64, i64, i64, i32, P(f64), P(i32), P(i32))
_declare('tt_R_symbol', i32, i64, i64, i32, P(f64), P(i32), P(i32))
_declare('tt_leg', i32, i32, P(i64), P(i64), P(i32))
_declare('tt_leg_blocks', i32, i32, P(i64), P(i64), P(i32))
_declare('tt_reachable_charges', i32, i32, P(i32), i32, P(i64), P(i32))
_declare('tt_fusion_trees', i32, i32, P(i32), i64, i64, P(i64), P(i64), P(i32))
_declare('tt_space', i32, i32, P(i32), i32, P(i32), i64, P(i32))
_declare('tt_space_size', i32, P(i64), P(i64))
_declare('tt_space_blocks', i32, i64, P(i64), P(i64))
_declare('tt_space_legs', i32, i32, P(i32), P(i32), P(i32), P(i64))
_declare('tt_plan_place', i32, i32, P(i32), i32, P(i32), P(vp))
_declare('tt_plan_conj', i32, P(vp))
_declare('tt_plan_contract', i32, i32, i32, P(i32), P(i32), i32, i64, P(vp))
_declare('tt_plan_einsum', ctypes.c_char_p, i32, P(i32), i32, i64, P(vp))
_declare('tt_plan_info', vp, P(i32), P(i64), P(f64), P(i64), P(i32))
_declare('tt_plan_prepared_size', vp, i32, P(i64))
_declare('tt_plan_describe', vp, i64, ctypes.c_char_p, P(i64))
_declare('tt_plan_cache_clear')
_declare('tt_plan_gather', vp, i32, i64, P(i32), P(i64))
_declare('tt_plan_execute', vp, i32, i32, P(vp), P(vp), vp, vp, vp)
_declare('tt_plan_execute_batch', i32, P(vp), i32, i32, P(vp), P(vp), P(vp), P(vp), vp, P(i32))
_declare('tt_plan_execute_timed', vp, i32, i32, P(vp), P(vp), vp, vp, vp, i32, P(ctypes.c_float), P(i32))
_declare('tt_plan_prepare', vp, i32, i32, vp, vp, vp, vp)
_declare('tt_step_plan', i32, i32, i32, i64, i64, i32, i64, P(i64), i64, P(f64), P(i64), P(i64))
_declare('tt_chain', i32, i32, P(i32), i32, P(i32), i32, P(i32), P(i32))
_declare('tt_dots', i32, i32, vp, vp, i64, vp, vp, vp)
_declare('tt_dots_noalloc', i32, i32, vp, vp, i64, vp, vp)
_declare('tt_svd_workspace', i32, P(i64), P(i64), P(i64))
_declare('tt_lanczos_scratch', i64, i32, i32, P(i64))
_declare('tt_lanczos', vp, i32, i32, P(vp), P(vp), i32, vp, i32, f64, vp, vp, vp, P(f64), P(i32), vp)
_declare('tt_lanczos_async', vp, i32, i32, P(vp), P(vp), i32, vp, i32, f64, vp, vp, vp, P(f64), P(i32), vp)
_declare('tt_plan_histogram', vp, P(ctypes.c_uint64))
_declare('tt_autotune', vp, i32, i32, P(vp), P(vp), vp, vp, vp, P(i32), P(ctypes.c_float))
_declare('tt_autotune_lookup', ctypes.c_uint64, i32, i32, P(i32), P(i32))
_declare('tt_autotune_store', ctypes.c_uint64, i32, i32, i32)
_declare('tt_autotune_clear')
_declare('tt_link_copy', vp, vp, i64, i32, vp)
_declare('tt_svd_rank', vp, i32, vp, vp, i32, vp, i32, f64, i64, vp, vp)
_declare('tt_svd_blocks', i32, i64, vp, vp, vp, vp, vp, vp, vp, vp)
_declare('tt_svd_keep', i32, vp, vp, vp, vp, vp, vp, vp, vp)

_ERRORS = {1: ValueError, 2: IndexError, 3: RuntimeError, 4: RuntimeError}


def check(status):
    '''Raise the exception a failed call maps to.'''
    if status != 0:
        message = lib.tt_last_error().decode()
        raise _ERRORS.get(status, RuntimeError)(message)


def ints32(values):
    values = list(values)
    return (i32 * max(len(values), 1))(*values), len(values)


def ints64(values):
    values = list(values)
    return (i64 * max(len(values), 1))(*values), len(values)


def pointers(values):
    values = list(values)
    return (vp * max(len(values), 1))(*values)


EXPORTED = ['tt_last_error', 'tt_version', 'tt_category', 'tt_outcomes', 'tt_dual', 'tt_q_dim', 'tt_F_symbol',
            'tt_R_symbol', 'tt_leg', 'tt_leg_blocks', 'tt_reachable_charges', 'tt_fusion_trees', 'tt_space',
            'tt_space_size', 'tt_space_blocks', 'tt_space_legs', 'tt_plan_place', 'tt_plan_conj', 'tt_plan_contract', 'tt_plan_einsum',
            'tt_plan_info', 'tt_plan_describe', 'tt_plan_cache_clear', 'tt_plan_gather', 'tt_plan_prepared_size', 'tt_plan_execute', 'tt_plan_execute_timed', 'tt_plan_prepare', 'tt_step_plan', 'tt_chain', 'tt_svd_workspace', 'tt_lanczos_scratch', 'tt_lanczos', 'tt_svd_blocks', 'tt_svd_keep',
            'tt_dots', 'tt_dots_noalloc', 'tt_plan_execute_batch', 'tt_lanczos_async', 'tt_plan_histogram', 'tt_autotune',
            'tt_autotune_lookup', 'tt_autotune_store', 'tt_autotune_clear', 'tt_link_copy', 'tt_svd_rank']
