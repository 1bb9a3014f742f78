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

from . import _lib, h5
from .pipelines import (CheckTraces, Clip, FilterTraces, GradientDescent, MaskField, MuteTraces, NormField,
                        NormPerShot, SmoothField, apply_prec)

__all__ = ['PlainFWI', 'LearnedFWI', 'relative_error', 'features', 'generate_pairs', 'train_unet', 'run_to_error',
           'dump_state', 'load_state']


def dump_state(vp, history, inner, spacing, path, project_name='fwi'):
    """Per-iteration dump for restarts, as the reference's inversion loop keeps them
    (stride/__init__.py:281-297, optimisation_loop.py:475-530): the model as a vp field file
    ``<project>-Vp[-%05d].h5`` whose version is the number of completed iterations (the
    reference's ScalarField description: inner ``data`` and its grid, plus ``extended_data`` so
    that the absorbing frame is restored exactly), and the loop's per-iteration records in
    ``<project>-OptimisationLoop.h5``."""
    vp = np.ascontiguousarray(vp, dtype=np.float32)
    inner_shape = tuple(s.stop - s.start for s in inner)
    extra = tuple(s.start for s in inner)
    desc = {'space': {'shape': inner_shape, 'spacing': tuple(float(h) for h in spacing), 'extra': extra,
                      'absorbing': extra},
            'shape': inner_shape, 'extended_shape': vp.shape,
            'inner': [[str(s.start), str(s.stop), 'None'] for s in inner], 'dtype': 'float32',
            'data': np.ascontiguousarray(vp[inner]), 'extended_data': vp, 'time_dependent': False}
    version = len(history)
    with h5.HDF5(project_name=project_name, parameter='vp', path=path, version=version, mode='w') as f:
        f.dump(desc)
    loop = {'num_iterations': version,
            'iterations': [dict({'id': k}, **{key: rec[key] for key in ('misfit', 'error', 'seconds', 'f_max')})
                           for k, rec in enumerate(history)]}
    with h5.HDF5(project_name=project_name, parameter='optimisation_loop', path=path, version=0, mode='w') as f:
        f.dump(loop)
    return version


def load_state(path, project_name='fwi', version=None):
    """(extended vp, history records, version) of a dump: the latest model version unless one is
    given, and the loop records up to it."""
    with h5.HDF5(project_name=project_name, parameter='vp', path=path, version=version, mode='r') as f:
        d = f.load(lazy=False)
    vp = np.asarray(d['extended_data'] if 'extended_data' in d else d['data'], dtype=np.float32)
    with h5.HDF5(project_name=project_name, parameter='optimisation_loop', path=path, version=0, mode='r') as f:
        loop = f.load(lazy=False)
    recs = loop['iterations'] if loop.get('num_iterations', 0) > 0 else []
    done = len(recs) if version is None else int(version)
    history = [{key: r[key] for key in ('misfit', 'error', 'seconds', 'f_max')} for r in recs[:done]]
    return vp, history, len(history)


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

    def set_step_size(self, step_size):
        """The gradient-descent step (the reference's step_size)."""
        self.step_size = step_size
        self.optimiser = GradientDescent(step_size=step_size, slowness=True)

    def reset(self, vp_true, vp0=1500.):
        """A new true model on the same grid and acquisition: observed data recomputed, vp restarted."""
        self.vp_true = torch.as_tensor(np.ascontiguousarray(vp_true, np.float32), device=self.device)
        self.plan.set_medium(self.vp_true, self.rho, self.alpha)
        self.plan.forward((self.wavelets * self.win[None]).contiguous(), self.observed)
        self.vp.fill_(float(vp0))
        self.history = []

    def close(self):
        self.plan.close()

    def dump(self, path, project_name='fwi'):
        """Writes the current model and loop records (``dump_state``); returns the version."""
        return dump_state(self.vp.cpu().numpy(), self.history, self.inner, self.w['spacing'], path, project_name)

    def resume(self, path, project_name='fwi', version=None):
        """Restores the model and loop records of a dump (the latest unless ``version``); returns the
        number of completed iterations, from which ``iterate`` continues."""
        vp, history, done = load_state(path, project_name, version)
        if tuple(vp.shape) != tuple(self.vp.shape):
            raise ValueError('dumped model of shape %s on a grid of shape %s' % (vp.shape, tuple(self.vp.shape)))
        self.vp.copy_(torch.as_tensor(vp, device=self.device))
        self.history = history
        return done

    def error(self):
        return relative_error(self.vp, self.vp_true, self.inner)

    def _modelled(self, vp, f_max, save):
        dt = self.dt
        filt = FilterTraces(f_max=f_max)
        wav = filt.forward(self.check.forward(self.wavelets), dt=dt) if f_max else self.wavelets
        obs = filt.forward(self.check.forward(self.observed), dt=dt) if f_max else self.observed
        self.plan.set_medium(vp, self.rho, self.alpha)
        modelled = torch.zeros_like(self.observed)
        self.plan.forward((wav * self.win[None]).contiguous(), modelled, save=save)
        return modelled, obs

    def misfit(self, vp, f_max=None):
        """Misfit of a model (forward only, the same trace processing as the gradient)."""
        modelled, obs = self._modelled(vp, f_max, False)
        res, _ = self._residual(modelled, obs, f_max)
        return 0.5 * float((res.double() ** 2).sum())

    def _residual(self, modelled, obs, f_max):
        dt = self.dt
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
        return mod - obs, tfilt

    def gradient(self, f_max=None):
        """Misfit, and the raw slowness gradient and preconditioner of the current model."""
        dt = self.dt
        modelled, obs = self._modelled(self.vp, f_max, True)
        res, tfilt = self._residual(modelled, obs, f_max)
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
        """Processed update direction over the inner grid: the reference's gradient is the inner
        region of the plan's (get_grad_vp, iso_acoustic/devito.py:1062-1097; the buffers of
        Data.clear_grad, problem/data.py:352-372), so Data.apply_prec normalises by the inner
        points and MaskField ramps at the inner field's own edges, then smooth and norm (against
        the whole model, as NormField reads the variable's extended data)."""
        g, _ = apply_prec(grad[self.inner].contiguous(), prec[self.inner].contiguous())
        g = self.mask.forward(g, (slice(None),) * g.dim())
        g = self.smooth.forward(g)
        return self.normf.forward(g, variable=self.vp, transform=lambda x: 1 / x)

    def take_step(self, d):
        """The optimiser's update of the inner model (LocalOptimiser.update_variable on
        variable.data, optimisers/optimiser.py:273-298), then the clip of the whole model."""
        v = self.vp[self.inner].contiguous()
        self.optimiser.step(v, d)
        self.vp[self.inner] = v
        self.vp.copy_(self.clip.forward(self.vp))

    def iterate(self, f_max=None):
        t0 = time.perf_counter()
        misfit, grad, prec = self.gradient(f_max)
        self.take_step(self.direction(grad, prec))
        torch.cuda.synchronize(self.device)
        rec = dict(misfit=misfit, error=self.error(), seconds=time.perf_counter() - t0, f_max=f_max)
        self.history.append(rec)
        return rec


# ---- learned preconditioner -------------------------------------------------------------------

VP_REF, VP_SCALE = 1500., 100.  # network units: (vp - 1500) / 100 and vp updates / 100


def features(grad, vp, inner):
    """Network input [1, H, W, 2] on the inner grid: the raw slowness gradient scaled to max |g| = 1
    and (vp - 1500) / 100."""
    g = grad[inner]
    g = g / (g.abs().max() + 1e-30)
    v = (vp[inner] - VP_REF) / VP_SCALE
    return torch.stack([g, v], dim=-1)[None].contiguous()


class LearnedFWI(PlainFWI):
    """FWI whose update is the U-Net's prediction from [gradient, model], accepted only when the
    plain misfit decreases; otherwise the plain gradient step of ``PlainFWI`` is taken."""

    def __init__(self, w, net, **kwargs):
        super().__init__(w, **kwargs)
        self.net = net

    def iterate(self, f_max=None):
        t0 = time.perf_counter()
        misfit, grad, prec = self.gradient(f_max)
        x = features(grad, self.vp, self.inner)
        y = self.net.forward(x)
        H, W = x.shape[1], x.shape[2]
        dvp = self.net.output(y, 1, H, W)[0, ..., 0] * VP_SCALE
        cand = self.vp.clone()
        cand[self.inner] += dvp
        cand = self.clip.forward(cand)
        accepted = self.misfit(cand, f_max) < misfit
        if accepted:
            self.vp.copy_(cand)
        else:
            self.take_step(self.direction(grad, prec))
        torch.cuda.synchronize(self.device)
        rec = dict(misfit=misfit, error=self.error(), seconds=time.perf_counter() - t0, f_max=f_max,
                   learned=bool(accepted))
        self.history.append(rec)
        return rec


def generate_pairs(fwi, phantoms_vp, iterations=5, f_max=None):
    """Training pairs along plain-FWI paths: for each true model, ``iterations`` plain updates from
    the start model, each contributing (features(gradient, vp), (vp_true - vp) / 100)."""
    xs, ts = [], []
    for vp_true in phantoms_vp:
        fwi.reset(vp_true)
        for _ in range(iterations):
            _, grad, prec = fwi.gradient(f_max)
            xs.append(features(grad, fwi.vp, fwi.inner))
            ts.append(((fwi.vp_true - fwi.vp)[fwi.inner] / VP_SCALE)[None].contiguous())
            fwi.take_step(fwi.direction(grad, prec))
    return torch.cat(xs), torch.cat(ts)


def train_unet(net, X, T, epochs=20, batch=4, lr=1e-3, seed=0, graph=True):
    """Adam on the mean squared error of the predicted update; returns the per-epoch losses. With
    graph, every step replays one captured training step (unet.GraphTrainer), bit for bit the eager
    step."""
    from .unet import GraphTrainer
    g = torch.Generator(device='cpu').manual_seed(seed)
    n = X.shape[0]
    losses = []
    trainer = GraphTrainer(net, batch, X.shape[1], X.shape[2], X.shape[3], lr=lr) if graph and n >= batch else None
    for _ in range(epochs):
        perm = torch.randperm(n, generator=g)
        tot = 0.
        if trainer is not None:
            trainer.loss_sum.zero_()
        for i in range(0, n - batch + 1, batch):
            idx = perm[i:i + batch].to(X.device)
            if trainer is not None:
                trainer.train_step(X[idx], T[idx])
                continue
            y = net.forward(X[idx].contiguous())
            loss, d = net.mse(y, T[idx].contiguous())
            net.backward(d)
            net.adam_step(lr=lr)
            tot += float(loss.item())
        if trainer is not None:
            tot = float(trainer.loss_sum.item())
        losses.append(tot / max(1, n // batch))
    return losses


def run_to_error(fwi, vp_true, target, max_iter=30, f_max=None):
    """Iterates from the start model until the relative vp error is <= target; returns (wall
    seconds or None if not reached, iterations, errors)."""
    fwi.reset(vp_true)
    torch.cuda.synchronize(fwi.device)
    t0 = time.perf_counter()
    errs = [fwi.error()]
    if errs[0] <= target:
        return 0.0, 0, errs
    for it in range(max_iter):
        errs.append(fwi.iterate(f_max)['error'])
        if errs[-1] <= target:
            return time.perf_counter() - t0, it + 1, errs
    return None, max_iter, errs
