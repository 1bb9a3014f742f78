"""ctypes binding of libstrideacc.so (declared in include/strideacc.h).

The library is the only compute path: loading fails loudly when it has not been built
(``python -m stride_gb300.build`` or ``__graft_entry__.build()``); there is no CPU fallback.
"""

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, '_build', 'libstrideacc.so')

SA_OK = 0
SA_E_INVALID = -1
SA_E_UNSUPPORTED = -2
SA_E_CUDA = -3
SA_E_NOMEM = -4
SA_E_TIMEOUT = -5
SA_OPT_PERSISTENT = 1
SA_OPT_BARRIER_EXTRA = 2
SA_OPT_BARRIER_SPIN = 3

SA_KERNEL_OT2 = 2
SA_KERNEL_OT4 = 4
SA_DENSITY_NONE = 0
SA_DENSITY_VARIABLE = 1
SA_DENSITY_CONSTANT = 2
SA_SAVE_NONE = 0
SA_SAVE_SNAPSHOTS = 1
SA_SAVE_CHECKPOINTS = 2
SA_SAVE_RAW = 3
SA_GRAD_PARITY = 0
SA_BOUNDARY_SPONGE = 0
SA_BOUNDARY_CFS_PML = 1
SA_INTERP_LINEAR = 0
SA_INTERP_HICKS = 1
SA_INTERP_SINC = 2
SA_GRAD_EXACT = 1

# every symbol include/strideacc.h declares
EXPORTS = ('sa_plan_create', 'sa_plan_destroy', 'sa_set_medium', 'sa_set_geometry', 'sa_forward',
           'sa_adjoint', 'sa_adjoint_wavelets', 'sa_adjoint_grads', 'sa_autotune', 'sa_last_error', 'sa_launch_count',
           'sa_plan_layout', 'sa_plan_option', 'sa_checkpoint_schedule',
           'sa_forward_2d_noalloc',
           'sa_traces_sosfilt', 'sa_traces_fir', 'sa_traces_check', 'sa_traces_norm_per_shot', 'sa_traces_mute',
           'sa_field_mul', 'sa_field_clip', 'sa_field_axpy', 'sa_field_slowness_step', 'sa_field_stats',
           'sa_field_scale', 'sa_field_gaussian', 'sa_field_apply_prec', 'sa_gemm_bf16', 'sa_nn_im2col',
           'sa_nn_col2im', 'sa_nn_transpose_bf16', 'sa_nn_to_bf16', 'sa_nn_relu_bwd', 'sa_nn_bias_grad',
           'sa_nn_maxpool', 'sa_nn_maxpool_bwd', 'sa_nn_upsample', 'sa_nn_upsample_bwd', 'sa_nn_copy_channels',
           'sa_nn_pack_weights', 'sa_nn_adam', 'sa_nn_mse', 'sa_nn_sum_slabs', 'sa_conv3x3_bf16',
           'sa_nn_adam_corrections', 'sa_nn_adam_dev')


class SaDesc(ctypes.Structure):
    _fields_ = [('dim', ctypes.c_int), ('shape', ctypes.c_int * 3), ('spacing', ctypes.c_double * 3),
                ('extra', ctypes.c_int * 3), ('absorbing', ctypes.c_int * 3), ('dt', ctypes.c_double),
                ('nt', ctypes.c_int), ('kernel', ctypes.c_int), ('density', ctypes.c_int),
                ('attenuation', ctypes.c_int), ('undersampling', ctypes.c_int), ('max_shots', ctypes.c_int),
                ('checkpoint_interval', ctypes.c_int), ('checkpoint_budget', ctypes.c_double),
                ('interpolation', ctypes.c_int), ('boundary', ctypes.c_int), ('f_centre', ctypes.c_double)]


class StrideAccError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__('strideacc error %d: %s' % (code, msg))
        self.code = code


_lib = None


def load():
    """Loads the library (raises ImportError when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError('libstrideacc.so is not built (%s); run stride_gb300.build.build()' % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    I = ctypes.c_int
    lib.sa_plan_create.argtypes = [ctypes.POINTER(SaDesc), ctypes.POINTER(P)]
    lib.sa_plan_destroy.argtypes = [P]
    lib.sa_set_medium.argtypes = [P, P, P, P]
    lib.sa_set_geometry.argtypes = [P, I, P, P, P, P]
    lib.sa_forward.argtypes = [P, P, P, I, P]
    lib.sa_adjoint.argtypes = [P, P, P, P, I, P]
    lib.sa_adjoint_wavelets.argtypes = [P, P, P, P, P, I, P]
    lib.sa_adjoint_grads.argtypes = [P, P, P, P, P, P, P, P]
    lib.sa_autotune.argtypes = [P, P]
    lib.sa_last_error.argtypes = [ctypes.c_char_p, I]
    lib.sa_launch_count.argtypes = [P]
    lib.sa_launch_count.restype = ctypes.c_longlong
    IP = ctypes.POINTER(I)
    lib.sa_plan_layout.argtypes = [P, IP, IP, IP]
    lib.sa_plan_option.argtypes = [P, I, ctypes.c_longlong]
    lib.sa_checkpoint_schedule.argtypes = [ctypes.POINTER(SaDesc), I, IP, IP, IP]
    L = ctypes.c_longlong
    F = ctypes.c_float
    D = ctypes.c_double
    lib.sa_traces_sosfilt.argtypes = [P, P, I, I, P, I, I, P]
    lib.sa_traces_fir.argtypes = [P, P, I, I, P, I, I, I, P]
    lib.sa_traces_check.argtypes = [P, I, I, P, I, P]
    lib.sa_traces_norm_per_shot.argtypes = [P, P, P, I, I, P, P]
    lib.sa_traces_mute.argtypes = [P, P, P, I, I, P, I, P]
    lib.sa_field_mul.argtypes = [P, P, L, P]
    lib.sa_field_clip.argtypes = [P, L, P, P, P]
    lib.sa_field_axpy.argtypes = [P, P, L, F, P]
    lib.sa_field_slowness_step.argtypes = [P, P, L, F, P]
    lib.sa_field_stats.argtypes = [P, L, P, P, P]
    lib.sa_field_scale.argtypes = [P, L, D, P]
    lib.sa_field_gaussian.argtypes = [P, I, P, P, I, P, P]
    lib.sa_field_apply_prec.argtypes = [P, P, L, D, P]
    lib.sa_gemm_bf16.argtypes = [P, I, P, I, P, I, P, I, I, I, I, P, I, I, I, P, P]
    lib.sa_nn_im2col.argtypes = [P, I, I, I, I, I, P, I, P]
    lib.sa_nn_col2im.argtypes = [P, I, I, I, I, I, P, I, I, P]
    lib.sa_nn_transpose_bf16.argtypes = [P, I, I, I, P, I, I, P]
    lib.sa_nn_to_bf16.argtypes = [P, I, L, I, P, I, P]
    lib.sa_nn_relu_bwd.argtypes = [P, I, P, I, L, I, P]
    lib.sa_nn_bias_grad.argtypes = [P, I, L, I, P, P, P]
    lib.sa_nn_sum_slabs.argtypes = [P, L, I, P, L, I, P]
    lib.sa_conv3x3_bf16.argtypes = [P, I, I, I, I, I, P, I, P, I, P, I, I, I, P, I, P, P]
    lib.sa_nn_maxpool.argtypes = [P, I, I, I, I, I, P, I, P]
    lib.sa_nn_maxpool_bwd.argtypes = [P, I, P, I, I, I, I, I, P, I, I, P]
    lib.sa_nn_upsample.argtypes = [P, I, I, I, I, I, P, I, P]
    lib.sa_nn_upsample_bwd.argtypes = [P, I, I, I, I, I, P, I, P]
    lib.sa_nn_copy_channels.argtypes = [P, I, L, I, P, I, I, P]
    lib.sa_nn_pack_weights.argtypes = [P, I, I, P, P, I, I, P]
    lib.sa_nn_adam.argtypes = [P, P, P, P, L, F, F, F, F, I, P]
    lib.sa_nn_adam_corrections.argtypes = [F, F, I, P]
    lib.sa_nn_adam_dev.argtypes = [P, P, P, P, L, F, F, F, F, P, I, P, P]
    lib.sa_nn_mse.argtypes = [P, I, P, L, P, I, P, P]
    for name in EXPORTS:
        if name not in ('sa_launch_count',):
            getattr(lib, name).restype = I
    _lib = lib
    return lib


def checkpoint_schedule(dim, shape, nt, n_shots=1, undersampling=4, checkpoint_interval=0, checkpoint_budget=0.0,
                        boundary='sponge'):
    """(K, n_checkpoints, K2) that sa_forward(SA_SAVE_CHECKPOINTS) takes for n_shots shots: the
    coarse interval and count and the fine interval of a two-level schedule (0: one level). Host
    only; raises StrideAccError(SA_E_NOMEM) when nothing fits checkpoint_budget bytes."""
    d = SaDesc()
    d.dim = dim
    for i in range(3):
        d.shape[i] = int(shape[i]) if i < dim else 1
    d.nt = int(nt)
    d.undersampling = int(undersampling)
    d.checkpoint_interval = int(checkpoint_interval)
    d.checkpoint_budget = float(checkpoint_budget)
    d.boundary = {'sponge': SA_BOUNDARY_SPONGE, 'pml': SA_BOUNDARY_CFS_PML}[boundary]
    K, n, K2 = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    check(load().sa_checkpoint_schedule(ctypes.byref(d), int(n_shots), ctypes.byref(K), ctypes.byref(n),
                                        ctypes.byref(K2)))
    return K.value, n.value, K2.value


def last_error():
    buf = ctypes.create_string_buffer(512)
    load().sa_last_error(buf, 512)
    return buf.value.decode(errors='replace')


def check(code):
    if code != SA_OK:
        raise StrideAccError(code, last_error())


def _ptr(x):
    """Raw pointer of a numpy array or a torch tensor (None stays NULL)."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        if not x.flags['C_CONTIGUOUS']:
            raise ValueError('array must be C-contiguous')
        return x.ctypes.data_as(ctypes.c_void_p)
    if hasattr(x, 'data_ptr'):
        if not x.is_contiguous():
            raise ValueError('tensor must be contiguous')
        return ctypes.c_void_p(x.data_ptr())
    raise TypeError('unsupported buffer type %r' % type(x))


def _stream(stream):
    if stream is None:
        return None
    if hasattr(stream, 'cuda_stream'):
        return ctypes.c_void_p(stream.cuda_stream)
    return ctypes.c_void_p(int(stream))


class Plan:
    """Owner of one sa_plan (one batch of shots on one grid)."""

    def __init__(self, dim, shape, spacing, extra, absorbing, dt, nt, kernel='OT4', density=SA_DENSITY_NONE,
                 attenuation=False, undersampling=4, max_shots=1, checkpoint_interval=0, checkpoint_budget=0.0,
                 interpolation='linear', boundary='sponge', f_centre=0.0):
        """boundary: 'sponge' (SpongeBoundary2) or 'pml' (ComplexFrequencyShiftPML2, OT2, 2D and 3D, with
        the band centre f_centre in Hz)."""
        lib = load()
        d = SaDesc()
        d.dim = dim
        for i in range(3):
            d.shape[i] = int(shape[i]) if i < dim else 1
            d.spacing[i] = float(spacing[i]) if i < dim else 1.0
            d.extra[i] = int(extra[i]) if i < dim else 0
            d.absorbing[i] = int(absorbing[i]) if i < dim else 0
        d.dt = float(dt)
        d.nt = int(nt)
        d.kernel = SA_KERNEL_OT4 if kernel == 'OT4' else SA_KERNEL_OT2
        d.density = int(density)
        d.attenuation = int(bool(attenuation))
        d.undersampling = int(undersampling)
        d.max_shots = int(max_shots)
        d.checkpoint_interval = int(checkpoint_interval)
        d.checkpoint_budget = float(checkpoint_budget)
        d.interpolation = {'linear': SA_INTERP_LINEAR, 'hicks': SA_INTERP_HICKS, 'sinc': SA_INTERP_SINC}[interpolation]
        d.boundary = {'sponge': SA_BOUNDARY_SPONGE, 'pml': SA_BOUNDARY_CFS_PML}[boundary]
        d.f_centre = float(f_centre)
        self.desc = d
        h = ctypes.c_void_p()
        check(lib.sa_plan_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self.dim = dim
        self.nt = int(nt)
        self.n_src = 0
        self.n_rec = 0

    def close(self):
        if getattr(self, '_h', None) is not None and self._h.value:
            load().sa_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_medium(self, vp, rho=None, alpha=None):
        check(load().sa_set_medium(self._h, _ptr(vp), _ptr(rho), _ptr(alpha)))

    def set_geometry(self, src_offsets, src_xyz, rec_offsets, rec_xyz):
        so = np.ascontiguousarray(src_offsets, dtype=np.int32)
        ro = np.ascontiguousarray(rec_offsets, dtype=np.int32)
        sx = np.ascontiguousarray(src_xyz, dtype=np.float32).reshape(-1, self.dim)
        rx = np.ascontiguousarray(rec_xyz, dtype=np.float32).reshape(-1, self.dim)
        check(load().sa_set_geometry(self._h, len(so) - 1, _ptr(so), _ptr(sx), _ptr(ro), _ptr(rx)))
        self.n_src = int(so[-1])
        self.n_rec = int(ro[-1])

    def forward(self, wavelets, traces, save=False, stream=None):
        """save: False, True / 'snapshots' (p.dt2 every f steps), 'raw' (p itself every f steps,
        for the rho and wavelet gradients of the reference) or 'checkpoints'."""
        mode = {False: SA_SAVE_NONE, None: SA_SAVE_NONE, True: SA_SAVE_SNAPSHOTS, 'snapshots': SA_SAVE_SNAPSHOTS,
                'checkpoints': SA_SAVE_CHECKPOINTS, 'raw': SA_SAVE_RAW}[save]
        check(load().sa_forward(self._h, _ptr(wavelets), _ptr(traces), mode, _stream(stream)))

    def adjoint(self, residuals, grad, prec, stream=None, exact=False, grad_wavelets=None, grad_rho=None,
                prec_rho=None):
        """exact=False: the reference's imaging condition; exact=True: dL/dvp of the discrete forward
        map for residuals = dL/dtraces (needs a forward with save='checkpoints'). grad_wavelets
        [n_src, nt]: also the reference's wavelet gradient -interp(p_a) (parity mode).
        grad_rho/prec_rho [shape]: also the rho gradient (needs a forward with save='raw')."""
        if grad_rho is not None or prec_rho is not None:
            if exact:
                raise ValueError('the rho gradient is the reference imaging condition (exact=False)')
            check(load().sa_adjoint_grads(self._h, _ptr(residuals), _ptr(grad), _ptr(prec), _ptr(grad_rho),
                                          _ptr(prec_rho), _ptr(grad_wavelets), _stream(stream)))
            return
        check(load().sa_adjoint_wavelets(self._h, _ptr(residuals), _ptr(grad), _ptr(prec), _ptr(grad_wavelets),
                                         SA_GRAD_EXACT if exact else SA_GRAD_PARITY, _stream(stream)))

    def autotune(self, stream=None):
        check(load().sa_autotune(self._h, _stream(stream)))

    @property
    def launches(self):
        return int(load().sa_launch_count(self._h))

    def set_option(self, option, value):
        """sa_plan_option: SA_OPT_PERSISTENT, SA_OPT_BARRIER_EXTRA or SA_OPT_BARRIER_SPIN."""
        check(load().sa_plan_option(self._h, int(option), int(value)))

    @property
    def layout(self):
        """(threads per CTA, column strips, row chunks) of the time-step launches."""
        t, s, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(load().sa_plan_layout(self._h, ctypes.byref(t), ctypes.byref(s), ctypes.byref(c)))
        return t.value, s.value, c.value
