"""The C ABI: library present, every declared symbol exported, argument validation and the
error channel. No GPU: no call here reaches a kernel."""

import ctypes
import os
import re

import pytest

from stride_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, 'include', 'strideacc.h')).read()
    return sorted(set(re.findall(r'^(?:int|long long)\s+(sa_\w+)\s*\(', text, re.M)))


@pytest.fixture(scope='module')
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from stride_gb300 import build
        build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert names, 'no declarations parsed'
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_lib.EXPORTS)


def test_invalid_description_is_rejected_before_cuda(lib):
    d = _lib.SaDesc()
    d.dim = 5
    h = ctypes.c_void_p()
    rc = lib.sa_plan_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == _lib.SA_E_UNSUPPORTED
    assert 'dim' in _lib.last_error()
    d.dim = 2
    d.kernel = 3
    rc = lib.sa_plan_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == _lib.SA_E_INVALID and 'kernel' in _lib.last_error().lower()


def test_null_arguments(lib):
    assert lib.sa_plan_create(None, None) == _lib.SA_E_INVALID
    assert lib.sa_forward(None, None, None, 0, None) == _lib.SA_E_INVALID
    assert lib.sa_adjoint(None, None, None, None, 0, None) == _lib.SA_E_INVALID
    assert lib.sa_set_medium(None, None, None, None) == _lib.SA_E_INVALID
    assert lib.sa_plan_destroy(None) == _lib.SA_OK
    assert lib.sa_launch_count(None) == -1


def test_error_raises_in_python(lib):
    with pytest.raises(_lib.StrideAccError):
        _lib.Plan(4, (10, 10, 10), (1e-3,) * 3, (0,) * 3, (0,) * 3, 1e-7, 10)
