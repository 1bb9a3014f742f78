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


def test_noalloc_matches_allocating_forward_twice():
    import torch
    c = C.small_case(kernel='OT4', density='variable', alpha=True, n_shots=1)
    ref, plan = C.gpu_forward(c)  # sa_forward: the existing, allocating entry point
    ref = ref[0]
    fn = _noalloc(_lib.load())
    dev = torch.device('cuda', 0)
    nt = c['nt']
    vp = torch.from_numpy(np.ascontiguousarray(c['vp'])).to(dev)
    rho = torch.from_numpy(np.ascontiguousarray(c['rho'])).to(dev)
    alpha = torch.from_numpy(np.ascontiguousarray(c['alpha'])).to(dev)
    wav = np.tile((c['wav'] * C.window(nt))[None], (len(c['srcs'][0]), 1)).astype(np.float32)
    wav_d = torch.from_numpy(wav).to(dev)
    eps = (1e-3 * np.asarray(c['spacing'])).astype(np.float32)
    sx = np.ascontiguousarray(np.asarray(c['srcs'][0], np.float32) + eps)
    rx = np.ascontiguousarray(np.asarray(c['recs'][0], np.float32) + eps)
    traces = torch.zeros((len(rx), nt), device=dev)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    for call in range(2):
        traces.fill_(float('nan'))
        rc = fn(ctypes.byref(plan.desc), p(vp), p(rho), p(alpha), len(sx), sx.ctypes.data_as(ctypes.c_void_p),
                p(wav_d), len(rx), rx.ctypes.data_as(ctypes.c_void_p), p(traces), None)
        assert rc == _lib.SA_OK, _lib.last_error()
        torch.cuda.synchronize()
        got = traces.cpu().numpy()
        assert np.isfinite(got).all(), call
        assert C.rel_l2(got, ref) <= 1e-4, call


def test_noalloc_rejects_oversize_grids():
    fn = _noalloc(_lib.load())
    d = _lib.SaDesc()
    d.dim = 2
    d.shape[0] = d.shape[1] = 700
    d.nt = 10
    rc = fn(ctypes.byref(d), None, None, None, 0, None, None, 0, None, None, None)
    assert rc == _lib.SA_E_INVALID
    assert '640' in _lib.last_error()
