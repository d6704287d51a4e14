"""ctypes binding of the in-tree C-ABI library (``include/oopao_gb300.h``).

The library is the only compute path: there is no CPU fallback.  Loading
fails with an exception when the library has not been built, and every
status code other than OOPAO_OK raises ``OopaoError``.
"""
import ctypes
import os

from .tools import OopaoError

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, '_lib', 'liboopao_gb300.so')

c_int, c_float, c_double, c_size_t, c_void_p = (ctypes.c_int, ctypes.c_float, ctypes.c_double,
                                                 ctypes.c_size_t, ctypes.c_void_p)
P = ctypes.POINTER

# name -> (restype, argtypes); mirrors include/oopao_gb300.h
SIGNATURES = {
    'oopao_abi_version': (c_int, []),
    'oopao_last_error': (ctypes.c_char_p, []),
    'oopao_launch_count': (ctypes.c_ulonglong, []),
    'oopao_pwfs_plan_create': (c_int, [P(c_void_p), c_int, c_int, c_int, c_int, c_void_p, c_void_p,
                                       c_double, c_int]),
    'oopao_pwfs_plan_destroy': (c_int, [c_void_p]),
    'oopao_pwfs_set_amplitude': (c_int, [c_void_p, c_void_p]),
    'oopao_pwfs_set_weights': (c_int, [c_void_p, c_void_p]),
    'oopao_pwfs_set_masks': (c_int, [c_void_p, c_int, c_void_p]),
    'oopao_pwfs_n_masks': (c_int, [c_void_p]),
    'oopao_pwfs_set_launch': (c_int, [c_void_p, c_int, c_int, c_int, c_int]),
    'oopao_pwfs_set_pass_budget': (c_int, [c_void_p, c_size_t]),
    'oopao_pwfs_set_variant': (c_int, [c_void_p, c_int]),
    'oopao_pwfs_get_variant': (c_int, [c_void_p]),
    'oopao_pwfs_device_status': (c_int, [c_void_p, c_void_p]),
    'oopao_pwfs_num_variants': (c_int, [c_void_p]),
    'oopao_pwfs_variant_info': (c_int, [c_void_p, c_int, c_void_p]),
    'oopao_pwfs_set_separable': (c_int, [c_void_p, c_int]),
    'oopao_pwfs_separable': (c_int, [c_void_p]),
    'oopao_pwfs_num_separable': (c_int, [c_void_p]),
    'oopao_pwfs_pass_info': (c_int, [c_void_p, c_int, c_void_p]),
    'oopao_pwfs_workspace_bytes': (c_size_t, [c_void_p, c_int]),
    'oopao_pwfs_measure': (c_int, [c_void_p, c_void_p, c_double, c_int, c_void_p, c_void_p, c_void_p,
                                   c_size_t, c_void_p]),
    'oopao_pwfs_measure_focal': (c_int, [c_void_p, c_void_p, c_double, c_int, c_void_p, c_void_p, c_void_p,
                                         c_void_p, c_size_t, c_void_p]),
    'oopao_pwfs_measure_noalloc':(c_int, [c_void_p, c_void_p, c_double, c_int, c_void_p, c_void_p, c_void_p]),
    'oopao_pwfs_set_profiling': (c_int, [c_void_p, c_int]),
    'oopao_pwfs_profile_read': (c_int, [c_void_p, c_void_p, c_void_p]),
    'oopao_pwfs_set_signal_processing': (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                                 c_double, c_double]),
    'oopao_pwfs_n_signal': (c_int, [c_void_p]),
    'oopao_pwfs_signal': (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    'oopao_dm_opd_f32': (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_float, c_void_p, c_void_p]),
    'oopao_dm_vjp_f32': (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_float, c_void_p, c_void_p]),
    'oopao_dm_opd_acc_f32': (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_float, c_void_p, c_void_p,
                                     c_void_p]),
    'oopao_dm_modes_bf16': (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p]),
    'oopao_dm_sep_workspace_bytes': (c_size_t, [c_int, c_int, c_int]),
    'oopao_dm_opd_sep_f32': (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p, c_int, c_int, c_int,
                                     c_float, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    'oopao_dm_bf16_workspace_bytes': (c_size_t, [c_int, c_int]),
    'oopao_dm_opd_bf16': (c_int, [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_float, c_void_p, c_void_p,
                                  c_void_p, c_size_t, c_void_p]),
    'oopao_dm_opd_bf16_tiled': (c_int, [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_float, c_void_p, c_void_p,
                                        c_void_p, c_size_t, c_int, c_void_p]),
    'oopao_cl_screen': (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_int, c_void_p, c_void_p, c_void_p]),
    'oopao_cl_integrate': (c_int, [c_void_p, c_void_p, c_int, c_int, c_float, c_void_p, c_void_p, c_void_p]),
    'oopao_cl_modal': (c_int, [c_void_p, c_void_p, c_int, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    'oopao_cl_pupil_rms': (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_int, c_void_p]),
    'oopao_atm_update': (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p,
                                 c_void_p, c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                                 c_void_p, c_int, c_void_p, c_void_p]),
    'oopao_atm_boil': (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                               c_int, c_void_p, c_void_p]),
    'oopao_pwfs_ad_workspace_bytes': (c_size_t, [c_void_p, c_int]),
    'oopao_pwfs_jvp': (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_double, c_int, c_void_p, c_void_p,
                               c_size_t, c_void_p]),
    'oopao_pwfs_vjp': (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_int, c_void_p, c_void_p, c_size_t,
                               c_void_p]),
    'oopao_pwfs_signal_jvp': (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    'oopao_pwfs_signal_vjp': (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p]),
    'oopao_gsc_plan_create': (c_int, [P(c_void_p), c_int, c_int, c_void_p]),
    'oopao_gsc_plan_destroy': (c_int, [c_void_p]),
    'oopao_gsc_workspace_bytes': (c_size_t, [c_void_p, c_int]),
    'oopao_gsc_set_basis': (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    'oopao_gsc_calibrate': (c_int, [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    'oopao_gsc_optical_gains': (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                        c_size_t, c_void_p]),
    'oopao_gsc_read': (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    'oopao_dm_modes_tf32x2': (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p]),
    'oopao_dm_tf32_workspace_bytes': (c_size_t, [c_int, c_int]),
    'oopao_dm_opd_tf32x3': (c_int, [c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_float, c_void_p, c_void_p,
                                    c_void_p, c_size_t, c_void_p]),
    'oopao_det_saturate': (c_int, [c_void_p, c_int, c_int, c_float, c_void_p, c_void_p]),
    'oopao_det_readout_tail': (c_int, [c_void_p, c_int, c_int, c_float, c_int, c_float, c_int, c_int, c_int,
                                       c_void_p, c_void_p, c_void_p]),
}

_lib = None


def load(path=LIB_PATH):
    """Load the library once (``OopaoError`` if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OopaoError('oopao_gb300 CUDA library not built (%s); run '
                         '`python -m oopao_gb300.build`' % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, what=''):
    if status != 0:
        msg = load().oopao_last_error().decode(errors='replace')
        raise OopaoError('%s failed (status %d): %s' % (what, status, msg))


def _arg(a):
    """Pointer for an array/tensor argument (the caller keeps `a` alive)."""
    if a is None:
        return None
    if hasattr(a, 'data_ptr'):
        if not a.is_contiguous():
            raise OopaoError('non-contiguous tensor passed to the C ABI')
        return a.data_ptr()
    if hasattr(a, 'ctypes') and hasattr(a, 'flags'):
        if not a.flags['C_CONTIGUOUS']:
            raise OopaoError('non-contiguous array passed to the C ABI')
        return a.ctypes.data
    return a


def call(name, *args):
    """Call a C-ABI entry point.  numpy arrays and torch tensors may be passed
    directly: they are referenced by `args` for the whole call, so their
    memory cannot be released while the library reads it."""
    lib = load()
    st = getattr(lib, name)(*[_arg(a) for a in args])
    if SIGNATURES[name][0] is c_int and name not in ('oopao_abi_version', 'oopao_pwfs_n_signal', 'oopao_pwfs_n_masks',
                                                     'oopao_pwfs_get_variant', 'oopao_pwfs_num_variants',
                                                     'oopao_pwfs_separable', 'oopao_pwfs_num_separable'):
        check(st, name)
    return st


def host(a, dtype):
    """C-contiguous host copy/view of `a` with the given dtype (hold the result
    in a variable until the call that uses it has returned)."""
    import numpy as np
    return np.ascontiguousarray(a, dtype=dtype)


def ptr(t):
    """Device address of a torch tensor (None -> NULL).  Host arrays are passed
    to ``call`` directly instead, so that they stay alive during the call."""
    if t is None:
        return None
    if hasattr(t, 'data_ptr'):
        return t.data_ptr()
    raise OopaoError('ptr() takes torch tensors; pass numpy arrays to call() directly')


def stream_handle(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream
