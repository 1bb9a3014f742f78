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


def _level_2d(nx, ny, n_shots):
    return (n_shots + 1) // 2 * nx * ((ny + 2 + 31) // 32 * 32) * 8  # pair-interleaved float2 levels


def test_checkpoint_schedule_one_and_two_levels(lib):
    """The schedule sa_forward(SA_SAVE_CHECKPOINTS) takes, on the host: the requested interval
    rounded to a multiple of f; under a budget, the nearest one-level interval that fits; below
    every one-level schedule, two levels with the largest fine interval that fits."""
    nt, f = 250, 4
    assert _lib.checkpoint_schedule(2, (60, 64), nt) == (52, 4, 0)
    assert _lib.checkpoint_schedule(2, (60, 64), nt, checkpoint_interval=30) == (32, 7, 0)
    L = _level_2d(60, 64, 3)
    one = lambda k, ck=2: ((nt - 2) // k) * ck * L + (k // f) * L
    two = lambda k1, k2, ck=2: ((nt - 2) // k1) * ck * L + (k1 // k2 - 1) * ck * L + (k2 // f) * L
    least = min(one(k) for k in range(f, nt - f, f))
    K, n, K2 = _lib.checkpoint_schedule(2, (60, 64), nt, n_shots=3, checkpoint_interval=40,
                                        checkpoint_budget=0.9 * least)
    assert (K, n, K2) == (96, 2, 48)  # the schedule the two-level GPU test runs
    assert K % K2 == 0 and K2 % f == 0 and two(K, K2) <= 0.9 * least
    K, n, K2 = _lib.checkpoint_schedule(2, (60, 64), nt, n_shots=3, checkpoint_interval=40,
                                        checkpoint_budget=1.5 * least)
    assert K2 == 0 and one(K) <= 1.5 * least
    # the CFS-PML's auxiliary fields make each checkpoint eight levels: under a budget the sponge's
    # requested interval fits, the PML's does not, and a longer one is taken
    budget = 2.5 * least
    assert _lib.checkpoint_schedule(2, (60, 64), nt, n_shots=3, checkpoint_interval=40,
                                    checkpoint_budget=budget)[0] == 40
    K, n, K2 = _lib.checkpoint_schedule(2, (60, 64), nt, n_shots=3, checkpoint_interval=40,
                                        checkpoint_budget=budget, boundary='pml')
    assert one(40, 8) > budget and K2 == 0 and K > 40 and one(K, 8) <= budget
    with pytest.raises(_lib.StrideAccError) as e:  # eight-level checkpoints need at least 32 levels here
        _lib.checkpoint_schedule(2, (60, 64), nt, n_shots=3, checkpoint_budget=1.5 * least, boundary='pml')
    assert e.value.code == _lib.SA_E_NOMEM
    with pytest.raises(_lib.StrideAccError) as e:
        _lib.checkpoint_schedule(2, (60, 64), nt, n_shots=3, checkpoint_budget=2 * L)
    assert e.value.code == _lib.SA_E_NOMEM
    # 3D: one level of every shot, z padded to 32
    L3 = 2 * 40 * 42 * 64 * 4
    K, n, K2 = _lib.checkpoint_schedule(3, (40, 42, 45), 130, n_shots=2, checkpoint_interval=40,
                                        checkpoint_budget=0.9 * min(((128) // k) * 2 * L3 + (k // f) * L3
                                                                    for k in range(f, 126, f)))
    assert (K, K2) == (72, 36)
    with pytest.raises(_lib.StrideAccError):
        _lib.checkpoint_schedule(4, (1, 1, 1), 10)
