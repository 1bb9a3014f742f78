"""GPU trace and field processing: the optimisation-pipeline steps on either side of a gradient.

Mirrors Stride's steps (stride/optimisation/pipelines/steps/*.py, stride/problem/data.py
``apply_prec``, the gradient-descent update of stride/optimisation/optimisers/optimiser.py) with
the same names, options and forward/adjoint behaviour, on CUDA tensors: traces are
``[n_traces, nt]`` float32 (``Traces.extended_data``), fields float32 on the extended grid. The
arithmetic runs in libstrideacc.so (``stride_gb300/csrc/pipelines.cu``); filter design
(``scipy.signal.butter`` / ``firwin``, the cosine table, Gaussian taps) is host set-up, as in the
reference.
"""

import numpy as np
import scipy.signal
import torch

from . import _lib

__all__ = ['FilterTraces', 'NormPerShot', 'NormPerTrace', 'MuteTraces', 'CheckTraces', 'MaskField',
           'SmoothField', 'NormField', 'Clip', 'apply_prec', 'GradientDescent', 'rampoff_mask']


def _stream():
    return _lib._stream(torch.cuda.current_stream())


def _check_traces_tensor(x):
    if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.float32 and x.dim() == 2):
        raise TypeError('traces must be a 2D float32 CUDA tensor [n_traces, nt]')
    return x.contiguous()


def _check_field(x):
    if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.float32):
        raise TypeError('fields must be float32 CUDA tensors')
    return x.contiguous()


def _cos_table(filter_length):
    # _make_filter_cos (stride/utils/filters.py:400-410)
    i = np.arange(1, filter_length + 1)
    table = 1. - np.cos(2 * np.pi * i / (filter_length + 1))
    return table / np.sum(table)


class FilterTraces:
    """FilterTraces (optimisation/pipelines/steps/filter_traces.py): lowpass (``cos`` by default),
    highpass or bandpass (``butterworth`` by default) in dimensionless frequency f * dt, causal
    (zero_phase=False as the step calls the filters), ``fir`` on request; the adjoint filters the
    time-reversed traces."""

    def __init__(self, f_min=None, f_max=None, filter_type=None, filter_relaxation=1.0, order=8, attenuation=30):
        self.f_min = f_min
        self.f_max = f_max
        self.filter_type = filter_type
        self.relaxation = filter_relaxation
        self.order = order
        self.attenuation = attenuation
        self._num_traces = None
        self._cache = {}

    def forward(self, *traces, dt, **kwargs):
        self._num_traces = len(traces)
        out = tuple(self._apply(t, dt, False, **kwargs) for t in traces)
        return out if len(out) > 1 else out[0]

    def adjoint(self, *d_traces, dt, **kwargs):
        d_traces = d_traces[:self._num_traces]
        out = tuple(self._apply(t, dt, True, **kwargs) for t in d_traces)
        self._num_traces = None
        return out if len(out) > 1 else out[0]

    def _design(self, dt, f_min, f_max, relaxation, ftype):
        key = (dt, f_min, f_max, relaxation, ftype)
        if key in self._cache:
            return self._cache[key]
        lo = relaxation * f_min * dt if f_min is not None else 0
        hi = 1 / relaxation * f_max * dt if f_max is not None else 0
        band = 'lowpass' if f_min is None else ('highpass' if f_max is None else 'bandpass')
        if ftype == 'butterworth':
            wn = {'lowpass': hi / 0.5, 'highpass': lo / 0.5, 'bandpass': [lo / 0.5, hi / 0.5]}[band]
            sos = scipy.signal.butter(self.order, wn, analog=False, btype={'bandpass': 'band'}.get(band, band),
                                      output='sos')
            design = ('sos', np.ascontiguousarray(sos, np.float64))
        elif ftype == 'cos':
            if band != 'lowpass':
                raise Exception('Requested filter does not exist. Implemented filters are butterworth, fir & cos.')
            period = int(np.round(1 / (hi / 0.5)))
            taps = torch.as_tensor(_cos_table(2 * period + 1), dtype=torch.float64, device='cuda')
            design = ('fir', taps, 2 * period)
        elif ftype == 'fir':
            order, beta = scipy.signal.kaiserord(self.attenuation, 0.050)
            order = order // 2 * 2 + 1
            cutoff = {'lowpass': hi / 0.5, 'highpass': lo / 0.5, 'bandpass': [lo / 0.5, hi / 0.5]}[band]
            b = scipy.signal.firwin(order, cutoff, pass_zero=band, window=('kaiser', beta), scale=True)
            taps = torch.as_tensor(np.ascontiguousarray(b[::-1]), dtype=torch.float64, device='cuda')
            design = ('fir', taps, len(b) - 1)  # lfilter(b, 1): y[t] = sum_k b[k] x[t - k]
        else:
            raise Exception('Requested filter does not exist. Implemented filters are butterworth, fir & cos.')
        self._cache[key] = design
        return design

    def _apply(self, traces, dt, adjoint, **kwargs):
        x = _check_traces_tensor(traces)
        f_min = kwargs.get('f_min', self.f_min)
        f_max = kwargs.get('f_max', self.f_max)
        relaxation = kwargs.get('filter_relaxation', self.relaxation)
        if f_min is None and f_max is None:
            return x.clone()
        ftype = kwargs.get('filter_type', self.filter_type or ('cos' if f_min is None else 'butterworth'))
        design = self._design(dt, f_min, f_max, relaxation, ftype)
        n, nt = x.shape
        out = torch.empty_like(x)
        lib = _lib.load()
        if design[0] == 'sos':
            sos = design[1]
            _lib.check(lib.sa_traces_sosfilt(_lib._ptr(x), _lib._ptr(out), n, nt, _lib._ptr(sos), sos.shape[0],
                                             int(adjoint), _stream()))
        else:
            taps, center = design[1], design[2]
            _lib.check(lib.sa_traces_fir(_lib._ptr(x), _lib._ptr(out), n, nt, _lib._ptr(taps), taps.numel(), center,
                                         int(adjoint), _stream()))
        return out


class NormPerShot:
    """NormPerShot (optimisation/pipelines/steps/norm_traces.py): each shot's traces divided by
    sqrt(sum of squares / trace count) + 1e-31; the adjoint passes the traces through, as the
    reference's does. ``offsets``: CSR trace offsets of the shots in a batch (default: one shot)."""

    def __init__(self, **kwargs):
        self._num_traces = None

    def forward(self, *traces, offsets=None, **kwargs):
        self._num_traces = len(traces)
        out = tuple(self._apply(t, offsets) for t in traces)
        return out if len(out) > 1 else out[0]

    def adjoint(self, *d_traces, **kwargs):
        d_traces = d_traces[:self._num_traces]
        return d_traces if len(d_traces) > 1 else d_traces[0]

    @staticmethod
    def _apply(traces, offsets):
        x = _check_traces_tensor(traces)
        n, nt = x.shape
        off = torch.as_tensor(np.asarray([0, n] if offsets is None else offsets, np.int32), device=x.device)
        scratch = torch.empty(len(off) - 1, dtype=torch.float64, device=x.device)
        out = torch.empty_like(x)
        _lib.check(_lib.load().sa_traces_norm_per_shot(_lib._ptr(x), _lib._ptr(out), _lib._ptr(off), len(off) - 1,
                                                       nt, _lib._ptr(scratch), _stream()))
        return out


class NormPerTrace(NormPerShot):
    """NormPerTrace (optimisation/pipelines/steps/norm_traces.py:72-88): every trace its own shot."""

    @staticmethod
    def _apply(traces, offsets):
        n = traces.shape[0]
        return NormPerShot._apply(traces, np.arange(n + 1))


class MuteTraces:
    """MuteTraces (optimisation/pipelines/steps/mute_traces.py): modelled traces multiplied by the
    cosine-lowpassed non-zero pattern of the observed ones; the adjoint passes through."""

    def __init__(self, f_max=None, filter_relaxation=1, **kwargs):
        self.f_max = f_max
        self.filter_relaxation = filter_relaxation
        self._num_traces = None

    def forward(self, modelled, observed, dt, **kwargs):
        self._num_traces = 2
        m = _check_traces_tensor(modelled)
        o = _check_traces_tensor(observed)
        f_max = kwargs.get('f_max', self.f_max)
        relax = kwargs.get('filter_relaxation', self.filter_relaxation)
        f = f_max * dt / relax if f_max is not None else 0.5
        period = int(np.round(1 / (f / 0.5)))
        taps = torch.as_tensor(_cos_table(2 * period + 1), dtype=torch.float64, device=m.device)
        out = torch.empty_like(m)
        n, nt = m.shape
        _lib.check(_lib.load().sa_traces_mute(_lib._ptr(m), _lib._ptr(o), _lib._ptr(out), n, nt, _lib._ptr(taps),
                                              taps.numel(), _stream()))
        return out, observed

    def adjoint(self, *d_traces, **kwargs):
        d_traces = d_traces[:self._num_traces]
        return d_traces if len(d_traces) > 1 else d_traces[0]


class CheckTraces:
    """CheckTraces (optimisation/pipelines/steps/check_traces.py): RuntimeError on NaN/inf traces
    (or a warning with raise_incorrect=False), optionally zeroing them."""

    def __init__(self, raise_incorrect=True, filter_incorrect=False, **kwargs):
        self.raise_incorrect = raise_incorrect
        self.filter_incorrect = filter_incorrect

    def forward(self, traces, name='traces', shot_id=None, **kwargs):
        x = _check_traces_tensor(traces).clone()
        n, nt = x.shape
        flags = torch.empty(max(n, 1), dtype=torch.int32, device=x.device)
        filt = kwargs.get('filter_incorrect', self.filter_incorrect)
        _lib.check(_lib.load().sa_traces_check(_lib._ptr(x), n, nt, _lib._ptr(flags), int(bool(filt)), _stream()))
        if n and bool(flags[:n].any()):
            msg = 'Nan or inf detected in %s' % name
            if shot_id is not None:
                msg = '(ShotID %d) ' % shot_id + msg
            if kwargs.get('raise_incorrect', self.raise_incorrect):
                raise RuntimeError(msg)
            import logging
            logging.getLogger('stride_gb300').warning(msg)
        return x

    def adjoint(self, d_traces, **kwargs):
        return d_traces


def rampoff_mask(shape, ramp_size):
    """_rampoff_mask (optimisation/pipelines/steps/mask_field.py:8-33), its index quirks kept
    (host set-up of the mask; the multiplication runs on the GPU)."""
    mask = np.ones(shape, dtype=np.float32)
    for dim_i in range(len(shape)):
        if 2 * ramp_size > shape[dim_i]:
            continue
        for index in range(ramp_size):
            pos = np.abs((ramp_size - index - 1) / float(ramp_size - 1))
            val = 1 - np.cos(np.pi / 2 * (1 - pos))
            all_ind = [slice(index, s - index + 1) for s in shape]
            all_ind[dim_i] = index
            mask[tuple(all_ind)] = val
            all_ind = [slice(index, s - index + 1) for s in shape]
            all_ind[dim_i] = -index
            mask[tuple(all_ind)] = val
    return mask


class MaskField:
    """MaskField (optimisation/pipelines/steps/mask_field.py): zero outside the inner domain, with a
    cosine ramp of ``mask_rampoff`` cells."""

    def __init__(self, mask_rampoff=10, mask=None, **kwargs):
        self.mask_rampoff = mask_rampoff
        self._mask = mask

    def forward(self, field, inner, **kwargs):
        x = _check_field(field).clone()
        mask = kwargs.get('mask', None)
        mask = self._mask if mask is None else mask
        if mask is None or tuple(mask.shape) != tuple(x.shape):
            m = np.zeros(tuple(x.shape), dtype=np.float32)
            m[inner] = 1
            m *= rampoff_mask(m.shape, kwargs.get('mask_rampoff', self.mask_rampoff))
            mask = torch.as_tensor(m, device=x.device)
            self._mask = mask
        mask = torch.as_tensor(mask, dtype=torch.float32, device=x.device).contiguous()
        _lib.check(_lib.load().sa_field_mul(_lib._ptr(x), _lib._ptr(mask), x.numel(), _stream()))
        return x


class SmoothField:
    """SmoothField (optimisation/pipelines/steps/smooth_field.py): Gaussian, 'nearest' borders."""

    def __init__(self, smooth_sigma=0.25, **kwargs):
        self.sigma = smooth_sigma

    def forward(self, field, **kwargs):
        x = _check_field(field)
        sigma = kwargs.get('smooth_sigma', self.sigma)
        if not np.iterable(sigma):
            sigma = (sigma,) * x.dim()
        if all(s <= 0 for s in sigma):
            return x
        return _gaussian(x.clone(), sigma, border=0)


def _gaussian(x, sigma, border):
    shape = np.asarray(x.shape, np.int32)
    sig = np.asarray(sigma, np.float64)
    scratch = torch.empty_like(x)
    _lib.check(_lib.load().sa_field_gaussian(_lib._ptr(x), x.dim(), _lib._ptr(shape), _lib._ptr(sig), border,
                                             _lib._ptr(scratch), _stream()))
    return x


def _stats(x):
    out = np.zeros(4, np.float32)
    s = np.zeros(1, np.float64)
    _lib.check(_lib.load().sa_field_stats(_lib._ptr(x), x.numel(), _lib._ptr(out), _lib._ptr(s), _stream()))
    return float(out[0]), float(out[1]), float(out[2]), float(s[0])


class NormField:
    """NormField (optimisation/pipelines/steps/norm_field.py): scale to max |x| = mid(variable) *
    norm_guess_change / 100 (1 without a variable)."""

    def __init__(self, global_norm=False, norm_guess_change=0.5, **kwargs):
        self.global_norm = global_norm
        self.norm_guess_change = norm_guess_change
        self.norm_value = None

    def forward(self, field, variable=None, transform=None, **kwargs):
        x = _check_field(field).clone()
        global_norm = kwargs.get('global_norm', self.global_norm)
        change = kwargs.get('norm_guess_change', self.norm_guess_change)
        if self.norm_value is None or not global_norm:
            self.norm_value = np.float32(_stats(x)[2]) + np.float32(1e-31)
        if variable is not None:
            vmin, vmax, _, _ = _stats(_check_field(variable))
            mid = (np.float32(vmax) + np.float32(vmin)) / 2.0
            if transform is not None:
                mid = transform(mid)
            var_corr = mid * change / 100
            var_corr = var_corr if np.abs(var_corr) > 0. else 1.
        else:
            var_corr = 1.
        scale = np.float32(var_corr / self.norm_value)
        _lib.check(_lib.load().sa_field_scale(_lib._ptr(x), x.numel(), float(scale), _stream()))
        return x


class Clip:
    """Clip (optimisation/pipelines/steps/clip.py)."""

    def __init__(self, min=None, max=None, **kwargs):  # noqa: A002 - the reference's argument names
        self.min = min
        self.max = max

    def forward(self, field, **kwargs):
        x = _check_field(field).clone()
        lo = None if self.min is None else np.asarray([self.min], np.float32)
        hi = None if self.max is None else np.asarray([self.max], np.float32)
        _lib.check(_lib.load().sa_field_clip(_lib._ptr(x), x.numel(), _lib._ptr(lo), _lib._ptr(hi), _stream()))
        return x


def apply_prec(grad, prec, prec_scale=4.0, prec_smooth=1.0):
    """Data.apply_prec (stride/problem/data.py:411-446): smooth the preconditioner ('reflect'
    Gaussian), scale it to prec_scale * N / sum|prec| and add 1, divide the gradient by it.
    Returns (grad, prec) as new tensors."""
    g = _check_field(grad).clone()
    p = _check_field(prec).clone()
    if prec_smooth is not None:
        sig = prec_smooth if np.iterable(prec_smooth) else (prec_smooth,) * p.dim()
        p = _gaussian(p, sig, border=1)
    sum_abs = _stats(p)[3]
    if sum_abs > 1e-31:
        factor = prec_scale * p.numel() / sum_abs
        _lib.check(_lib.load().sa_field_apply_prec(_lib._ptr(g), _lib._ptr(p), g.numel(), float(factor), _stream()))
    return g, p


class GradientDescent:
    """Gradient descent of a vp variable in slowness (optimisers/gradient_descent.py with the update
    of optimisers/optimiser.py:273-298 and the vp variable's slowness transform): vp <- 1 / (1/vp -
    step * direction). ``slowness=False`` updates vp itself."""

    def __init__(self, step_size=1., slowness=True):
        self.step_size = step_size
        self.slowness = slowness

    def step(self, vp, direction, step_size=None):
        v = _check_field(vp)
        d = _check_field(direction)
        step = self.step_size if step_size is None else step_size
        lib = _lib.load()
        if self.slowness:
            _lib.check(lib.sa_field_slowness_step(_lib._ptr(v), _lib._ptr(d), v.numel(), float(step), _stream()))
        else:
            _lib.check(lib.sa_field_axpy(_lib._ptr(v), _lib._ptr(d), v.numel(), float(-step), _stream()))
        return v
