"""Spectral helpers of the host path, following stride/utils/fft.py:8-141."""

import numpy as np

__all__ = ['magnitude_spectrum', 'bandwidth']


def magnitude_spectrum(signal, dt, db=True):
    """Magnitude of the one-sided spectrum (norm='forward'), optionally in dB re the peak."""
    num = signal.shape[-1]
    freqs = np.fft.rfftfreq(num, dt)
    mag = np.abs(np.fft.rfft(signal, axis=-1, norm='forward'))
    if db:
        mag = 20 * np.log10((mag + 1e-31) / (np.max(mag) + 1e-31))
    return freqs, mag


def bandwidth(signal, dt, cutoff=-10):
    """(f_min, f_centre, f_max) of the band above ``cutoff`` dB; multi-trace input uses the
    mean spectrum."""
    freqs, mag = magnitude_spectrum(signal, dt, db=True)
    if mag.ndim > 1:
        mag = np.mean(mag, axis=0)
    num = mag.shape[-1]
    f_min = 0
    for f in range(num):
        if mag[f] > cutoff:
            f_min = freqs[f]
            break
    f_centre = freqs[np.argmax(mag)]
    f_max = num
    for f in reversed(range(num)):
        if mag[f] > cutoff:
            f_max = freqs[f]
            break
    return f_min, f_centre, f_max
