"""Source wavelets (host side), following stride/utils/wavelets.py:6-53."""

import numpy as np
import scipy.signal

__all__ = ['tone_burst']


def tone_burst(centre_freq, n_cycles, n_samples, dt, envelope='gaussian', offset=0):
    """Tone burst of ``n_cycles`` at ``centre_freq`` with a Gaussian (+-3 sigma) or
    rectangular envelope, a 5 % Tukey taper, zero-padded to ``n_samples``."""
    tone_length = n_cycles / centre_freq
    t = np.linspace(0, tone_length, int(tone_length // dt + 1), endpoint=False)
    signal = np.sin(2 * np.pi * centre_freq * t)
    n_tone = signal.shape[0]
    if envelope == 'gaussian':
        window = np.exp(-np.linspace(-3, 3, n_tone) ** 2 / 2)
    elif envelope == 'rectangular':
        window = np.ones((n_tone,))
    else:
        raise Exception('Envelope type not implemented')
    signal = signal * window * scipy.signal.get_window(('tukey', 0.05), n_tone, False)
    return np.pad(signal, ((offset, n_samples - offset - n_tone),), mode='constant', constant_values=0.)
