"""Generates the golden fixtures of tests/golden (run: python tests/golden/make_golden.py).

analytic_2d.npz: the analytic 2D Green's-function traces of the reference's homogeneous
  example (stride_examples/examples/homogeneous_acoustic/utils.py:5-33, restated: wavelet
  derivative convolved with H(t - r/c) / (2 pi c^2 sqrt(t^2 - r^2/c^2))), normalised, for a
  500 kHz 3-cycle burst in 1500 m/s water, plus the same kernel integrated exactly over each
  sample (acosh form), which resolves the 1/sqrt singularity.
analytic_3d.npz: the 3D counterpart (utils.py:36-59): F(t - r/c) / (4 pi c^2 r).
oracle_small.npz: NumPy-oracle traces, snapshots checksum and vp gradient of a small
  variable-density, attenuating OT4 case: a regression fixture for the restatement.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import numpy_oracle as O  # noqa: E402


def ring(n, radius, centre):
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    return np.stack([radius * np.cos(ang) + centre[0], radius * np.sin(ang) + centre[1]], 1)


def analytic_2d(src, recs, wavelet, dt, nt, sos):
    wd = np.gradient(wavelet, dt)
    k = 1 / (2 * np.pi * sos ** 2)
    tg = np.linspace(0, dt * (nt - 1), nt)
    ref = np.zeros((len(recs), nt))
    exact = np.zeros((len(recs), nt))
    te = np.arange(nt + 1) * dt
    for i, rl in enumerate(recs):
        r = np.sqrt(np.sum((src - rl) ** 2))
        tau = int(np.round(r / (sos * dt)))
        if tau >= 0 and nt - tau > 0:
            h = np.zeros(nt)
            h[tau] = k
            with np.errstate(invalid='ignore', divide='ignore'):
                h[tau + 1:] = k / np.sqrt(tg[tau + 1:] ** 2 - r ** 2 / sos ** 2)
            ref[i] = np.convolve(h, wd * dt, mode='full')[:nt]
        if r > 0:
            T = r / sos
            C = np.where(te > T, np.arccosh(np.maximum(te / T, 1.0)), 0.0)
            exact[i] = np.convolve(k * np.diff(C), wd, mode='full')[:nt]
    return ref, exact


def analytic_3d(src, recs, wavelet, dt, nt, sos, h):
    wd = np.gradient(wavelet, dt)
    k = 1 / (4 * np.pi * sos ** 2)
    out = np.zeros((len(recs), nt))
    for i, rl in enumerate(recs):
        r = np.sqrt(np.sum((src - rl) ** 2))
        tau = int(np.round(r / (sos * dt)))
        if tau >= 0 and nt - tau > 0:
            kk = k / r if r > 0 else k * 2.66 / h
            hh = np.zeros(nt)
            hh[tau] = kk
            out[i] = np.convolve(hh, wd * dt, mode='full')[:nt]
    return out


def main():
    # 2D homogeneous case (the reference example's 0.5 mm / 0.08 us / 500 kHz, reduced grid)
    n, extra, h, dt, nt = 160, 20, 0.5e-3, 0.08e-6, 1000
    lim = h * (n - 1)
    geo = ring(16, (lim - 15e-3) / 2, (lim / 2, lim / 2))
    wav = O.tone_burst(0.5e6, 3, nt, dt)
    ref, exact = analytic_2d(geo[0], geo, wav, dt, nt, 1500.)
    np.savez_compressed(os.path.join(HERE, 'analytic_2d.npz'), n=n, extra=extra, h=h, dt=dt, nt=nt,
                        geometry=geo, wavelet=wav, reference_formula=ref, exact_integral=exact)
    # 3D homogeneous case
    n3, e3, dt3, nt3 = 48, 10, 0.06e-6, 500
    lim3 = h * (n3 - 1)
    c3 = np.array([lim3 / 2] * 3)
    src3 = c3 + np.array([-6e-3, 0, 0])
    recs3 = np.stack([c3 + np.array([6e-3, 0, 0]), c3 + np.array([0, 7e-3, 0]), c3 + np.array([3e-3, -5e-3, 4e-3])])
    wav3 = O.tone_burst(0.5e6, 3, nt3, dt3)
    an3 = analytic_3d(src3, recs3, wav3, dt3, nt3, 1500., h)
    np.savez_compressed(os.path.join(HERE, 'analytic_3d.npz'), n=n3, extra=e3, h=h, dt=dt3, nt=nt3,
                        src=src3, recs=recs3, wavelet=wav3, analytic=an3)
    # small regression case for the restatement
    rng = np.random.default_rng(7)
    shape = (40, 44)
    vp = (1500 + 120 * rng.random(shape)).astype(np.float32)
    rho = (1000 + 80 * rng.random(shape)).astype(np.float32)
    al = (0.5 * rng.random(shape)).astype(np.float32)
    hh = (0.5e-3, 0.5e-3)
    dts = 0.6 * hh[0] / 1650
    nts = 160
    e = 8
    origin = (-e * hh[0], -e * hh[1])
    src = np.array([[6e-3, 7e-3]])
    rec = np.array([[3e-3, 10e-3], [9e-3, 4e-3], [7.3e-3, 8.1e-3]])
    w = O.tone_burst(1.0e6, 3, nts, dts)[None]
    tr, snaps = O.forward(vp, hh, dts, nts, (e, e), src, rec, w, origin, rho=rho, alpha=al, save=True)
    res = tr * 0.5
    g, p = O.adjoint(vp, hh, dts, nts, (e, e), rec, res, origin, snaps, rho=rho, alpha=al)
    np.savez_compressed(os.path.join(HERE, 'oracle_small.npz'), vp=vp, rho=rho, alpha=al, h=hh, dt=dts, nt=nts,
                        extra=e, src=src, rec=rec, wavelet=w, traces=tr, grad=g, prec=p,
                        snap_sum=np.float64(np.sum(snaps, dtype=np.float64)))
    print('golden fixtures written to', HERE)


if __name__ == '__main__':
    main()
