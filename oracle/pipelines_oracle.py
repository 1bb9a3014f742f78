"""NumPy/SciPy oracle of the trace and field processing steps (test infrastructure only).

Restates, in the reference's own arithmetic (NumPy and SciPy, which the reference calls
directly), the optimisation-pipeline steps that the GPU kernels of
``stride_gb300/csrc/pipelines.cu`` replace. Imported only by ``tests/``; the product path never
calls it. Paths are relative to the reference repository root.
"""

import numpy as np
import scipy.ndimage
import scipy.signal


def cos_table(filter_length):
    """_make_filter_cos (stride/utils/filters.py:400-410)."""
    i = np.arange(1, filter_length + 1)
    table = 1. - np.cos(2 * np.pi * i / (filter_length + 1))
    return table / np.sum(table)


def lowpass_filter_cos(data, f_max, order=1, zero_phase=True, adjoint=False, axis=-1):
    """stride/utils/filters.py:413-465 (f_max dimensionless)."""
    f_max = f_max / 0.5
    period = int(np.round(1 / f_max))
    table = cos_table(2 * period + 1)
    if adjoint:
        data = np.flip(data, axis=axis)
    if not zero_phase:
        pad = [(0, 0)] * data.ndim
        pad[axis] = (period, 0)
        data = np.pad(data, pad, mode='constant', constant_values=0.)
    out = data
    for _ in range(order):
        out = scipy.ndimage.convolve1d(out, table, mode='constant', axis=axis)
    if not zero_phase:
        out = out.take(range(0, out.shape[-1] - period), axis=-1)
    if adjoint:
        out = np.flip(out, axis=axis)
    return out


def butterworth(data, band, f_min=None, f_max=None, order=8, adjoint=False):
    """band/low/highpass_filter_butterworth with zero_phase=False (stride/utils/filters.py:14-170)."""
    if band == 'bandpass':
        sos = scipy.signal.butter(order, [f_min / 0.5, f_max / 0.5], analog=False, btype='band', output='sos')
    elif band == 'lowpass':
        sos = scipy.signal.butter(order, f_max / 0.5, analog=False, btype='lowpass', output='sos')
    else:
        sos = scipy.signal.butter(order, f_min / 0.5, analog=False, btype='highpass', output='sos')
    if adjoint:
        data = np.flip(data, axis=-1)
    out = scipy.signal.sosfilt(sos, data, axis=-1)
    if adjoint:
        out = np.flip(out, axis=-1)
    return out


def filter_traces(traces, dt, f_min=None, f_max=None, filter_type=None, relaxation=1.0, adjoint=False):
    """FilterTraces._apply (optimisation/pipelines/steps/filter_traces.py:57-96) on FP32 traces."""
    lo = relaxation * f_min * dt if f_min is not None else 0
    hi = 1 / relaxation * f_max * dt if f_max is not None else 0
    if f_min is None and f_max is None:
        return traces.copy()
    ftype = filter_type or ('cos' if f_min is None else 'butterworth')
    if f_min is None:
        out = lowpass_filter_cos(traces, hi, zero_phase=False, adjoint=adjoint) if ftype == 'cos' else \
            butterworth(traces, 'lowpass', f_max=hi, adjoint=adjoint)
    elif f_max is None:
        out = butterworth(traces, 'highpass', f_min=lo, adjoint=adjoint)
    else:
        out = butterworth(traces, 'bandpass', f_min=lo, f_max=hi, adjoint=adjoint)
    return np.asarray(out).astype(np.float32)


def norm_per_shot(traces):
    """NormPerShot._apply (optimisation/pipelines/steps/norm_traces.py:43-69)."""
    norm_value = 0.
    for index in range(traces.shape[0]):
        norm_value += np.sum(traces[index] ** 2)
    norm_value = np.sqrt(norm_value / traces.shape[0]) + 1e-31
    return traces / norm_value


def mute_traces(modelled, observed, dt, f_max=None, filter_relaxation=1):
    """MuteTraces.forward (optimisation/pipelines/steps/mute_traces.py:25-57)."""
    mask = np.ones(observed.shape)
    mask[np.abs(observed) == 0.] = 0.
    f = f_max * dt / filter_relaxation if f_max is not None else 0.5
    mask = lowpass_filter_cos(mask, f_max=f, zero_phase=True, axis=-1)
    out = np.empty_like(modelled)
    out[:] = mask * modelled
    return out


def rampoff_mask(shape, ramp_size):
    """_rampoff_mask (optimisation/pipelines/steps/mask_field.py:8-33), its index quirks kept."""
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


def field_mask(extended_shape, inner, mask_rampoff=10):
    """MaskField's mask (optimisation/pipelines/steps/mask_field.py:52-66)."""
    mask = np.zeros(extended_shape, dtype=np.float32)
    mask[inner] = 1
    mask *= rampoff_mask(mask.shape, mask_rampoff)
    return mask


def smooth_field(field, sigma=0.25):
    """SmoothField.forward (optimisation/pipelines/steps/smooth_field.py:27-47)."""
    if not np.iterable(sigma):
        sigma = (sigma,) * field.ndim
    if all(s <= 0 for s in sigma):
        return field
    return scipy.ndimage.gaussian_filter(field, sigma=sigma, mode='nearest')


def norm_field(field, variable=None, norm_guess_change=0.5, transform=None):
    """NormField.forward (optimisation/pipelines/steps/norm_field.py:24-52), global_norm=False."""
    norm_value = np.max(np.abs(field)) + 1e-31
    if variable is not None:
        mid_val = (np.max(variable) + np.min(variable)) / 2.0
        if transform is not None:
            mid_val = transform(mid_val)
        var_corr = mid_val * norm_guess_change / 100
        var_corr = var_corr if np.abs(var_corr) > 0. else 1.
    else:
        var_corr = 1.
    out = field.copy()
    out *= var_corr / norm_value
    return out


def apply_prec(grad, prec, prec_scale=4.0, prec_smooth=1.0):
    """Data.apply_prec (stride/problem/data.py:411-446); returns (grad, prec)."""
    grad = grad.copy()
    prec = prec.copy()
    if prec_smooth is not None:
        prec[:] = scipy.ndimage.gaussian_filter(prec, prec_smooth)
    prec_factor = np.sum(np.abs(prec))
    if prec_factor > 1e-31:
        num_points = np.prod(prec.shape)
        prec_factor = prec_scale * num_points / prec_factor
        prec[:] = prec * prec_factor + 1
        non_zero = np.abs(prec) > 0.
        grad[non_zero] *= 1 / prec[non_zero]
    return grad, prec
