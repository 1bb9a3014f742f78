"""sa_forward_2d_noalloc, the entry point that allocates no device memory, against sa_forward.

Callers that cannot let a library allocate GPU memory (an application whose memory pool owns
the whole device, or a loop that must not pay the device-wide synchronisation of cudaFree)
use sa_forward_2d_noalloc: it runs the same time-step kernel with its scratch in a fixed
__device__ array of the library. This test calls it through the C ABI twice in a row on the
same inputs and compares each result with the traces of the allocating entry point
(relative L2 <= 1e-4, the tolerance of the trace parity tests). It sits in its own file,
collected last, so a run that stops at the first failure has run every other test before it.
"""

import ctypes

import numpy as np
import pytest

from stride_gb300 import _lib
from tests import _cases as C

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    P = ctypes.c_void_p
    fn = lib.sa_forward_2d_noalloc
    fn.argtypes = [ctypes.POINTER(_lib.SaDesc), P, P, P, ctypes.c_int, P, P, ctypes.c_int, P, P, P]
    fn.restype = ctypes.c_int
    return fn


def _inputs(c, dev):
    import torch
    nt = c['nt']
    to = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    wav = np.tile((c['wav'] * C.window(nt))[None], (len(c['srcs'][0]), 1)).astype(np.float32)
    eps = (1e-3 * np.asarray(c['spacing'])).astype(np.float32)
    sx = np.ascontiguousarray(np.asarray(c['srcs'][0], np.float32) + eps)
    rx = np.ascontiguousarray(np.asarray(c['recs'][0], np.float32) + eps)
    return to(c['vp']), to(c['rho']), to(c['alpha']), to(wav), sx, rx


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize('kernel', ['OT2', 'OT4'])
@pytest.mark.parametrize('density', ['none', 'constant', 'variable'])
def test_noalloc_matches_allocating_forward_twice(kernel, density):
    """Two calls in a row against sa_forward on the same inputs, for both time schemes and every
    density mode (the no-alloc path has its own layout and medium preparation for each)."""
    import torch
    c = C.small_case(kernel=kernel, density=density, alpha=density == 'variable', n_shots=1)
    ref, plan = C.gpu_forward(c)  # sa_forward: the existing, allocating entry point
    ref = ref[0]
    assert np.abs(ref).max() > 0
    fn = _noalloc(_lib.load())
    dev = torch.device('cuda', 0)
    vp, rho, alpha, wav_d, sx, rx = _inputs(c, dev)
    traces = torch.zeros((len(rx), c['nt']), device=dev)
    for call in range(2):
        traces.fill_(float('nan'))
        rc = fn(ctypes.byref(plan.desc), _ptr(vp), _ptr(rho), _ptr(alpha), len(sx),
                sx.ctypes.data_as(ctypes.c_void_p), _ptr(wav_d), len(rx), rx.ctypes.data_as(ctypes.c_void_p),
                _ptr(traces), None)
        assert rc == _lib.SA_OK, _lib.last_error()
        torch.cuda.synchronize()
        got = traces.cpu().numpy()
        assert np.isfinite(got).all(), call
        assert C.rel_l2(got, ref) <= 1e-4, call


def test_noalloc_without_sources_or_receivers():
    """No receivers: nothing to record, the call still succeeds. No sources: the field stays zero,
    so every trace is zero."""
    import torch
    c = C.small_case(kernel='OT4', density='none', n_shots=1, nt=120)
    _, plan = C.gpu_forward(c)
    fn = _noalloc(_lib.load())
    dev = torch.device('cuda', 0)
    vp, _, _, wav_d, sx, rx = _inputs(c, dev)
    rc = fn(ctypes.byref(plan.desc), _ptr(vp), None, None, len(sx), sx.ctypes.data_as(ctypes.c_void_p), _ptr(wav_d),
            0, None, None, None)
    assert rc == _lib.SA_OK, _lib.last_error()
    traces = torch.full((len(rx), c['nt']), float('nan'), device=dev)
    rc = fn(ctypes.byref(plan.desc), _ptr(vp), None, None, 0, None, None, len(rx), rx.ctypes.data_as(ctypes.c_void_p),
            _ptr(traces), None)
    assert rc == _lib.SA_OK, _lib.last_error()
    torch.cuda.synchronize()
    assert torch.count_nonzero(traces).item() == 0


def test_noalloc_rejects_device_coordinates():
    import torch
    c = C.small_case(kernel='OT4', density='none', n_shots=1, nt=60)
    _, plan = C.gpu_forward(c)
    fn = _noalloc(_lib.load())
    dev = torch.device('cuda', 0)
    vp, _, _, wav_d, sx, rx = _inputs(c, dev)
    sx_d = torch.from_numpy(sx).to(dev)
    traces = torch.zeros((len(rx), c['nt']), device=dev)
    rc = fn(ctypes.byref(plan.desc), _ptr(vp), None, None, len(sx), _ptr(sx_d), _ptr(wav_d), len(rx),
            rx.ctypes.data_as(ctypes.c_void_p), _ptr(traces), None)
    assert rc == _lib.SA_E_INVALID
    assert 'host pointers' in _lib.last_error()


def test_noalloc_rejects_oversize_grids():
    fn = _noalloc(_lib.load())
    d = _lib.SaDesc()
    d.dim = 2
    d.shape[0] = d.shape[1] = 700
    d.nt = 10
    rc = fn(ctypes.byref(d), None, None, None, 0, None, None, 0, None, None, None)
    assert rc == _lib.SA_E_INVALID
    assert '640' in _lib.last_error()
