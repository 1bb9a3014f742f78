"""ctypes wrapper of the C/OpenMP oracle (oracle/fdtd_oracle.c). Test infrastructure only.

The host-side preparation (damping profile, interpolation weights, Tukey windows,
attenuation units) reuses the NumPy restatement in oracle/numpy_oracle.py, which
follows stride/physics/iso_acoustic/devito.py:220-513 and 689-873; the time loop
runs in C. Parity against Devito is unpinned (see numpy_oracle's header).
"""

import ctypes
import os
import subprocess

import numpy as np

from . import numpy_oracle as npo

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, '_build', 'libfdtd_oracle.so')
_lib = None


class OraDesc(ctypes.Structure):
    _fields_ = [('dim', ctypes.c_int), ('n', ctypes.c_int * 3), ('h', ctypes.c_double * 3),
                ('dt', ctypes.c_double), ('nt', ctypes.c_int), ('kernel', ctypes.c_int),
                ('rho_mode', ctypes.c_int), ('has_alpha', ctypes.c_int), ('f', ctypes.c_int),
                ('absorbing', ctypes.c_int * 3), ('nthreads', ctypes.c_int)]


def build():
    subprocess.check_call(['make', '-s', '-C', _HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        _lib.ora_forward.argtypes = [ctypes.POINTER(OraDesc), P, P, P, P, ctypes.c_int, P, P, P,
                                     ctypes.c_double, ctypes.c_int, P, P, P, ctypes.c_int, P]
        _lib.ora_adjoint.argtypes = [ctypes.POINTER(OraDesc), P, P, P, P, ctypes.c_int, P, P, P, P, P, P]
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _flat_corners(base, shape):
    dim = len(shape)
    offs = npo._corner_offsets(dim)
    idx = np.zeros((base.shape[0], len(offs)), dtype=np.int64)
    for c, off in enumerate(offs):
        flat = np.zeros(base.shape[0], dtype=np.int64)
        for d in range(dim):
            flat = flat * shape[d] + (base[:, d] + off[d])
        idx[:, c] = flat
    return np.ascontiguousarray(idx)


def _desc(vp, spacing, dt, nt, absorbing, kernel, rho, alpha, f, nthreads):
    d = OraDesc()
    d.dim = vp.ndim
    for i in range(3):
        d.n[i] = vp.shape[i] if i < vp.ndim else 1
        d.h[i] = spacing[i] if i < vp.ndim else 1.0
        d.absorbing[i] = absorbing[i] if i < vp.ndim else 0
    d.dt = dt
    d.nt = nt
    d.kernel = 4 if kernel == 'OT4' else 2
    rho_mode = 0
    if rho is not None:
        r32 = rho.astype(np.float32)
        rho_mode = 2 if np.isclose(np.min(r32), np.max(r32)) else 1
    d.rho_mode = rho_mode
    d.has_alpha = int(alpha is not None)
    d.f = f
    d.nthreads = nthreads
    return d


def _materials(vp, rho, alpha):
    vp32 = np.ascontiguousarray(vp, dtype=np.float32)
    rho32 = None if rho is None else np.ascontiguousarray(rho, dtype=np.float32)
    a32 = None
    if alpha is not None:
        a32 = np.ascontiguousarray((alpha.astype(np.float32).astype(np.float64) * npo.DB_TO_NEPER)
                                   .astype(np.float32))
    return vp32, rho32, a32


def forward(vp, spacing, dt, nt, absorbing, src_coords, rec_coords, wavelets, origin,
            rho=None, alpha=None, kernel=None, save=False, undersampling=4, diff_source=False,
            nthreads=0):
    """Same contract as numpy_oracle.forward (FP32 only)."""
    h = max(spacing)
    if kernel is None:
        kernel = npo.select_kernel(dt, h, float(np.max(vp)), vp.ndim)
    vp32, rho32, a32 = _materials(vp, rho, alpha)
    damp = np.ascontiguousarray(npo.damping_profile(vp.shape, spacing, absorbing, vp32, dt))
    eps = 1e-3 * np.asarray(spacing)
    sb, sw = npo.linear_stencil(np.asarray(src_coords, np.float32) + eps, origin, spacing)
    rb, rw = npo.linear_stencil(np.asarray(rec_coords, np.float32) + eps, origin, spacing)
    wav = np.asarray(wavelets, np.float64)
    if diff_source:
        wav = np.gradient(wav, dt, axis=-1)
    src = np.ascontiguousarray((wav.T * npo.tukey(nt)[:, None]).astype(np.float32))
    scale = 2 * dt * dt / h
    if not diff_source:
        scale /= dt
    d = _desc(vp, spacing, dt, nt, absorbing, kernel, rho, alpha, undersampling, nthreads)
    rec = np.zeros((nt, rb.shape[0]), dtype=np.float32)
    n_snap = (nt + undersampling) // undersampling + 1
    snaps = np.zeros((n_snap,) + vp.shape, dtype=np.float32) if save else None
    rc = lib().ora_forward(ctypes.byref(d), _ptr(vp32), _ptr(rho32), _ptr(a32), _ptr(damp),
                           sb.shape[0], _ptr(_flat_corners(sb, vp.shape)), _ptr(np.ascontiguousarray(sw)),
                           _ptr(src), scale, rb.shape[0], _ptr(_flat_corners(rb, vp.shape)),
                           _ptr(np.ascontiguousarray(rw)), _ptr(rec), int(save), _ptr(snaps))
    if rc != 0:
        raise MemoryError('C oracle allocation failed')
    return np.ascontiguousarray(rec.T), snaps


def adjoint(vp, spacing, dt, nt, absorbing, rec_coords, residual, origin, snaps,
            rho=None, alpha=None, kernel=None, undersampling=4, nthreads=0):
    """Same contract as numpy_oracle.adjoint (FP32 accumulation)."""
    h = max(spacing)
    if kernel is None:
        kernel = npo.select_kernel(dt, h, float(np.max(vp)), vp.ndim)
    vp32, rho32, a32 = _materials(vp, rho, alpha)
    damp = np.ascontiguousarray(npo.damping_profile(vp.shape, spacing, absorbing, vp32, dt))
    eps = 1e-3 * np.asarray(spacing)
    rb, rw = npo.linear_stencil(np.asarray(rec_coords, np.float32) + eps, origin, spacing)
    res = np.ascontiguousarray((np.asarray(residual, np.float64).T * npo.tukey(nt)[:, None]).astype(np.float32))
    d = _desc(vp, spacing, dt, nt, absorbing, kernel, rho, alpha, undersampling, nthreads)
    grad = np.zeros(vp.shape, dtype=np.float32)
    prec = np.zeros(vp.shape, dtype=np.float32)
    rc = lib().ora_adjoint(ctypes.byref(d), _ptr(vp32), _ptr(rho32), _ptr(a32), _ptr(damp),
                           rb.shape[0], _ptr(_flat_corners(rb, vp.shape)), _ptr(np.ascontiguousarray(rw)),
                           _ptr(res), _ptr(np.ascontiguousarray(snaps, dtype=np.float32)), _ptr(grad), _ptr(prec))
    if rc != 0:
        raise MemoryError('C oracle allocation failed')
    return grad, prec
