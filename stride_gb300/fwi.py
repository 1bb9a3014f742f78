"""Plain full-waveform inversion of vp on one GPU.

Restates Stride's inversion loop (``stride.adjoint`` in stride/__init__.py:117-381 with the
default pipelines of stride/optimisation/pipelines/default_pipelines.py, ``GradientDescent`` of
stride/optimisation/optimisers/optimiser.py and the example driver
stride_examples/examples/breast2D/02_script_inverse.py) with every shot of the acquisition in
one batched plan and every trace and field operation on the GPU:

  wavelets, observed  -> check, filter (f_max)                      (ProcessWavelets / ProcessObserved)
  forward (save)      -> modelled
  modelled, observed  -> check, mute, filter, norm per shot         (ProcessTraces)
  L2 misfit, residual -> adjoint of the trace steps -> windowed adjoint source
  adjoint             -> raw grad/prec -> slowness chain rule       (IsoAcousticDevito.get_grad_vp)
  gradient            -> apply_prec, mask, smooth, norm             (Data.apply_prec, ProcessGlobalGradient)
  update              -> slowness gradient step, clip               (GradientDescent, ProcessModelIteration)
"""

import time

import numpy as np
import scipy.signal
import torch

from . import _lib
from .pipelines import (CheckTraces, Clip, FilterTraces, GradientDescent, MaskField, MuteTraces, NormField,
                        NormPerShot, SmoothField, apply_prec)

__all__ = ['PlainFWI', 'relative_error']


def relative_error(vp, vp_true, inner):
    """||vp - vp_true||_2 / ||vp_true||_2 on the inner grid."""
    a = vp[inner].double()
    b = vp_true[inner].double()
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def _density(rho):
    if rho is None:
        return _lib.SA_DENSITY_NONE
    r = np.asarray(rho, np.float32)
    return _lib.SA_DENSITY_CONSTANT if np.isclose(r.min(), r.max()) else _lib.SA_DENSITY_VARIABLE


class PlainFWI:
    """vp inversion of a batch of 2D shots.

    ``w``: a workload dict (``stride_gb300.phantoms.workload``: extended-grid materials, geometry,
    wavelet, shots); rho and alpha are kept at their true values, vp starts at ``vp0``.
    Options follow the reference's defaults: step_size 10, clip [1400, 1700], mask ramp 10 cells,
    smoothing sigma 0.25 cells, norm_guess_change 0.5, mute, norm per shot.
    """

    def __init__(self, w, vp0=1500., step_size=10., clip=(1400., 1700.), mute=True, norm_per_shot=True,
                 kernel='OT4', device=None):
        self.w = w
        self.device = torch.device(device) if device is not None else torch.device('cuda', torch.cuda.current_device())
        dev = self.device
        self.nt = w['nt']
        self.dt = w['dt']
        shape = w['shape']
        e = w['extra']
        self.inner = tuple(slice(a, s - a) for a, s in zip(e, shape))
        n_shots = len(w['shots'])
        self.plan = _lib.Plan(2, shape, w['spacing'], w['extra'], w['absorbing'], w['dt'], self.nt, kernel=kernel,
                              density=_density(w['rho']), attenuation=w['alpha'] is not None, undersampling=4,
                              max_shots=n_shots)
        eps = 1e-3 * np.asarray(w['spacing'])
        so = np.cumsum([0] + [len(x) for x in w['src']])
        ro = np.cumsum([0] + [len(x) for x in w['rec']])
        self.rec_offsets = ro
        self.rho = None if w['rho'] is None else torch.as_tensor(w['rho'], device=dev)
        self.alpha = None if w['alpha'] is None else torch.as_tensor(w['alpha'], device=dev)
        self.vp_true = torch.as_tensor(w['vp'], device=dev)
        self.plan.set_medium(self.vp_true, self.rho, self.alpha)
        self.plan.set_geometry(so, (np.concatenate(w['src']) + eps).astype(np.float32), ro,
                               (np.concatenate(w['rec']) + eps).astype(np.float32))
        self.win = torch.as_tensor(scipy.signal.get_window(('tukey', 0.001), self.nt, False).astype(np.float32),
                                   device=dev)
        wav = np.tile(w['wavelet'][None].astype(np.float32), (self.plan.n_src, 1))
        self.wavelets = torch.as_tensor(wav, device=dev)
        self.observed = torch.zeros((self.plan.n_rec, self.nt), device=dev)
        self.plan.forward(self.wavelets * self.win[None], self.observed)
        self.vp = torch.full(shape, float(vp0), device=dev)
        self.step_size = step_size
        self.mute = MuteTraces() if mute else None
        self.norm = NormPerShot() if norm_per_shot else None
        self.check = CheckTraces()
        self.mask = MaskField()
        self.smooth = SmoothField()
        self.normf = NormField()
        self.clip = Clip(min=clip[0], max=clip[1])
        self.optimiser = GradientDescent(step_size=step_size, slowness=True)
        self.history = []

    def close(self):
        self.plan.close()

    def error(self):
        return relative_error(self.vp, self.vp_true, self.inner)

    def gradient(self, f_max=None):
        """Misfit, and the raw slowness gradient and preconditioner of the current model."""
        dt = self.dt
        filt = FilterTraces(f_max=f_max)
        wav = filt.forward(self.check.forward(self.wavelets), dt=dt) if f_max else self.wavelets
        obs = filt.forward(self.check.forward(self.observed), dt=dt) if f_max else self.observed
        self.plan.set_medium(self.vp, self.rho, self.alpha)
        modelled = torch.zeros_like(self.observed)
        self.plan.forward((wav * self.win[None]).contiguous(), modelled, save=True)
        mod = self.check.forward(modelled)
        if self.mute is not None:
            mod, _ = self.mute.forward(mod, obs, dt)
        tfilt = FilterTraces(f_max=f_max)
        if f_max:  # ProcessTraces filters both (the observed ones a second time, as the reference)
            mod = tfilt.forward(mod, dt=dt)
            obs = FilterTraces(f_max=f_max).forward(obs, dt=dt)
        if self.norm is not None:
            mod = self.norm.forward(mod, offsets=self.rec_offsets)
            obs = self.norm.forward(obs, offsets=self.rec_offsets)
        res = mod - obs
        misfit = 0.5 * float((res.double() ** 2).sum())
        # adjoint of the trace steps (norm and mute pass through, as the reference's)
        if f_max:
            res = tfilt.adjoint(res, dt=dt)
        adj = (res * self.win[None]).contiguous()
        grad = torch.zeros_like(self.vp)
        prec = torch.zeros_like(self.vp)
        self.plan.adjoint(adj, grad, prec)
        # get_grad_vp: slowness chain rule
        grad = grad / self.vp
        prec = prec / (self.vp * self.vp)
        return misfit, grad, prec

    def direction(self, grad, prec):
        """Processed update direction (Data.apply_prec, then mask / smooth / norm)."""
        g, _ = apply_prec(grad, prec)
        g = self.mask.forward(g, self.inner)
        g = self.smooth.forward(g)
        return self.normf.forward(g, variable=self.vp, transform=lambda x: 1 / x)

    def iterate(self, f_max=None):
        t0 = time.perf_counter()
        misfit, grad, prec = self.gradient(f_max)
        d = self.direction(grad, prec)
        self.optimiser.step(self.vp, d)
        self.vp.copy_(self.clip.forward(self.vp))
        torch.cuda.synchronize(self.device)
        rec = dict(misfit=misfit, error=self.error(), seconds=time.perf_counter() - t0, f_max=f_max)
        self.history.append(rec)
        return rec
