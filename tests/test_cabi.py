"""The C-ABI library loads and exports every symbol the public header declares
(no compute call: runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'oopao_gb300.h')


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r'/\*.*?\*/', '', txt, flags=re.S)
    return sorted(set(re.findall(r'\b(oopao_[a-z0-9_]+)\s*\(', txt)))


@pytest.fixture(scope='module')
def lib():
    from oopao_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert 'oopao_pwfs_measure' in syms and 'oopao_dm_opd_f32' in syms


def test_library_exports_declared_symbols(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    from oopao_gb300 import _native
    assert set(declared_symbols()) <= set(_native.SIGNATURES), \
        set(declared_symbols()) - set(_native.SIGNATURES)


def test_version_and_error_calls(lib):
    lib.oopao_abi_version.restype = ctypes.c_int
    assert lib.oopao_abi_version() >= 1
    lib.oopao_last_error.restype = ctypes.c_char_p
    assert isinstance(lib.oopao_last_error(), bytes)


def test_argument_validation_without_gpu(lib):
    """Invalid sizes are rejected on the host before any device work."""
    from oopao_gb300 import _native as N
    N.load()
    h = ctypes.c_void_p()
    # n_fft smaller than res
    st = N._lib.oopao_pwfs_plan_create(ctypes.byref(h), 32, 16, 8, 4, None, None, 1.0, 1)
    assert st == 1
    # prime factor 17 -> unsupported (checked before any allocation)
    import numpy as np
    mask = np.zeros((34, 34), np.complex64)
    path = np.zeros((4, 2))
    st = N._lib.oopao_pwfs_plan_create(ctypes.byref(h), 30, 34, 17, 4, mask.ctypes.data, path.ctypes.data, 1.0, 1)
    assert st == 2
    assert b'prime factor' in N._lib.oopao_last_error()
    # boiling: a one-step table without the step counter, layers out of order
    dummy = np.zeros(8)
    lay = np.array([1, 0], np.int32)
    ab = np.array([0.9, 0.4])
    f = N._lib.oopao_atm_boil
    f.argtypes = N.SIGNATURES['oopao_atm_boil'][1]
    st = f(dummy.ctypes.data, 2, 16, dummy.ctypes.data, 2, lay.ctypes.data, ab.ctypes.data, ab.ctypes.data, None, 2,
           None, None)
    assert st == 1 and b'step counter' in N._lib.oopao_last_error()
    st = f(dummy.ctypes.data, 2, 16, dummy.ctypes.data, 2, lay.ctypes.data, ab.ctypes.data, ab.ctypes.data, None, 1,
           None, None)
    assert st == 1 and b'increasing' in N._lib.oopao_last_error()
