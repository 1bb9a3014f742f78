"""Drop-in replacement of Stride's ``IsoAcousticDevito`` problem type on libstrideacc.

``IsoAcousticGB300`` keeps the reference's interface (stride/physics/iso_acoustic/devito.py):
the ``pde(wavelets, vp, rho=, alpha=, problem=, **kwargs)`` call through
``ProblemTypeBase.forward/adjoint`` (stride/physics/problem_type.py:58-112), the
before/run/after hooks, ``prepare/init/get_grad_vp``, the documented keyword arguments and
their error behaviour. The time loop runs in libstrideacc.so on the GPU (one plan per grid,
time axis and physics options); there is no CPU path.

When Stride is importable its ``ProblemTypeBase`` is the base class (and ``mosaic.tessera``
decorates the class as the reference's does), so Stride's scripts can swap the class in;
otherwise a local mirror of the base class is used.
"""

import logging
import time

import numpy as np
import scipy.signal

from . import _lib
from .fft import bandwidth

__all__ = ['IsoAcousticGB300', 'ProblemTypeBase']

try:  # pragma: no cover - Stride is not installed in the build container
    from stride.physics.problem_type import ProblemTypeBase as _StrideBase
    import mosaic as _mosaic
except Exception:  # noqa: BLE001
    _StrideBase = None
    _mosaic = None

DB_TO_NEPER = 100 * (1e-6 / (2 * np.pi)) ** 0 / (20 * np.log10(np.exp(1)))
PERF = 19  # the level of Devito's and Mosaic's 'perf' lines, between DEBUG and INFO
logging.addLevelName(PERF, 'PERF')

SUPPORTED_BOUNDARIES = ('sponge_boundary_2', 'complex_frequency_shift_PML_2')
KNOWN_BOUNDARIES = ('sponge_boundary_2', 'complex_frequency_shift_PML_2', 'sponge_boundary_1')
SUPPORTED_INTERPOLATION = ('linear', 'hicks', 'sinc')
KNOWN_INTERPOLATION = ('linear', 'hicks', 'sinc')


class _LocalProblemTypeBase:
    """Mirror of stride.physics.problem_type.ProblemTypeBase (problem_type.py:13-321):
    the forward/adjoint templates and the per-variable gradient dispatch."""

    def __init__(self, **kwargs):
        self.name = kwargs.pop('name', self.__class__.__name__.lower())
        grid = kwargs.get('grid', None)
        self.space = kwargs.get('space', getattr(grid, 'space', None))
        self.time = kwargs.get('time', getattr(grid, 'time', None))
        self.logger = logging.getLogger('stride_gb300')

    def forward(self, *args, **kwargs):
        self.before_forward(*args, **kwargs)
        out = self.run_forward(*args, **kwargs)
        res = self.after_forward(*args, **kwargs)
        return res if res is not None else out

    def __call__(self, *args, **kwargs):
        return self.forward(*args, **kwargs)

    def adjoint(self, *args, **kwargs):
        self.before_adjoint(*args, **kwargs)
        out = self.run_adjoint(*args, **kwargs)
        res = self.after_adjoint(*args, **kwargs)
        return res if res is not None else out

    def _dispatch(self, prefix, variable):
        methods = [getattr(self, prefix + tok, None) for tok in variable.name.split('_')]
        methods = [m for m in methods if m is not None]
        if not methods:
            raise ValueError('Variable %s not implemented' % variable.name)
        return methods[0]

    def prepare_grad(self, *wrt, **kwargs):
        updates = []
        for v in wrt:
            if v is None or not v.needs_grad:
                continue
            u = self._dispatch('prepare_grad_', v)(v, wrt=wrt, **kwargs)
            updates += list(u) if isinstance(u, tuple) else [u]
        return updates

    def init_grad(self, *wrt, **kwargs):
        for v in wrt:
            if v is None or not v.needs_grad:
                continue
            self._dispatch('init_grad_', v)(v, wrt=wrt, **kwargs)

    def get_grad(self, *wrt, **kwargs):
        grads = []
        for v in wrt:
            if v is None or not v.needs_grad:
                grads.append(None)
                continue
            g = self._dispatch('get_grad_', v)(v, wrt=wrt, **kwargs)
            gd = g.data if hasattr(g, 'data') else g
            if np.any(np.isnan(gd)) or np.any(np.isinf(gd)):
                problem = kwargs.get('problem', None)
                msg = 'Nan or inf detected in %s' % self.name
                if problem is not None:
                    msg = '(ShotID %d) ' % problem.shot.id + msg
                self.logger.warning(msg)
                return None
            grads.append(g)
        return tuple(grads)


ProblemTypeBase = _StrideBase if _StrideBase is not None else _LocalProblemTypeBase


def _tessera(cls):
    if _mosaic is not None:  # pragma: no cover
        return _mosaic.tessera(cls)
    return cls


@_tessera
class IsoAcousticGB300(ProblemTypeBase):
    """Second-order isotropic acoustic wave equation on the GB300 (forward, adjoint and vp
    gradient), with the keyword arguments of IsoAcousticDevito (devito.py:43-114).

    Supported: ``kernel`` OT2/OT4 (auto-selected from dt as the reference does),
    ``boundary_type='sponge_boundary_2'``, ``interpolation_type`` 'linear', 'hicks' or 'sinc',
    ``attenuation_power=0``, ``diff_source``, ``save_undersampling``, ``save_wavefield``.
    ``platform``, ``devito_config`` and ``devito_args`` are accepted and ignored (the time
    loop always runs on the GPU), and so is ``fw3d_mode``: the reference forces its fw3d adjoint
    injection on (devito.py:724-725), which is the one this class runs. ``boundary_type='complex_frequency_shift_PML_2'`` runs with
    kernel OT2 (the combination the reference's own example runs). Gradients: vp, rho and
    the wavelets; alpha raises ValueError('Variable alpha not implemented') as in the
    reference, which has no alpha gradient. Options the reference supports but this build does
    not (the CFS-PML with OT4, attenuation power 2) raise
    NotImplementedError; unknown values raise ValueError as in the reference.

    Memory: ``checkpoint_interval=K`` (steps) or ``checkpoint_budget`` (bytes) keeps the wavefield
    every K steps instead of every undersampled ``p.dt2`` and recomputes each segment in the
    adjoint; the vp gradient is the same, bit for bit. This stands where the reference reduces
    the saved wavefield with ``save_compression`` (devito.py:331-332), which is accepted and
    ignored. The raw-wavefield path (wavelet or rho gradients) always saves snapshots.
    """

    space_order = 10
    time_order = 2

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        self.kernel = 'OT4'
        self.drp = False
        self.undersampling_factor = 4
        self.boundary_type = 'sponge_boundary_2'
        self.interpolation_type = 'linear'
        self.attenuation_power = 0
        self.checkpoint_interval = 0
        self.checkpoint_budget = 0.0
        self._bandwidth = (0., 0., 0.)
        self._plans = {}
        self._plan = None
        self._saved = False
        self._grad = None
        self._prec = None
        self.logger = getattr(self, 'logger', logging.getLogger('stride_gb300'))

    # ---------------------------------------------------------------------------- checks

    def _perf(self, msg, *args):
        """A 'perf' line: Mosaic's logger level when the host logger has one, else PERF."""
        perf = getattr(self.logger, 'perf', None)
        if perf is not None:
            perf(msg % args if args else msg)
        else:
            self.logger.log(PERF, msg, *args)

    def _check_problem(self, wavelets, vp, rho=None, alpha=None, **kwargs):
        """Option validation and scheme selection (devito.py:1266-1352)."""
        boundary_type = kwargs.get('boundary_type', 'sponge_boundary_2')
        if not isinstance(boundary_type, str) or boundary_type not in KNOWN_BOUNDARIES:
            raise ValueError('Unknown boundary type %r' % (boundary_type,))
        if boundary_type not in SUPPORTED_BOUNDARIES:
            raise NotImplementedError('boundary_type %s is not implemented in this build' % boundary_type)
        self.boundary_type = boundary_type
        problem = kwargs.get('problem')
        self._perf('(ShotID %d) Selected boundary type %s', problem.shot.id if problem is not None else -1,
                   boundary_type)
        interpolation_type = kwargs.get('interpolation_type', self.interpolation_type)
        if interpolation_type not in KNOWN_INTERPOLATION:
            raise ValueError('Only "linear" and "hicks" interpolations are allowed.')
        if interpolation_type not in SUPPORTED_INTERPOLATION:
            raise NotImplementedError('interpolation_type %s is not implemented in this build' % interpolation_type)
        self.interpolation_type = interpolation_type
        attenuation_power = kwargs.get('attenuation_power', 0)
        if alpha is not None:
            if attenuation_power not in (0, 2, None):
                raise ValueError('The "attenuation_exponent" can only take values (0, 2).')
            if attenuation_power != 0:
                raise NotImplementedError('attenuation_power %r is not implemented in this build' % attenuation_power)
        self.attenuation_power = attenuation_power
        interval = kwargs.get('checkpoint_interval', 0) or 0
        budget = kwargs.get('checkpoint_budget', 0.0) or 0.0
        if int(interval) != interval or interval < 0 or budget < 0:
            raise ValueError('checkpoint_interval must be a non-negative integer and checkpoint_budget >= 0')
        self.checkpoint_interval, self.checkpoint_budget = int(interval), float(budget)
        if kwargs.get('drp', False):
            self.logger.warning('DRP weights are not implemented in this version of stride')
        self.drp = False
        self._check_conditions(wavelets, vp, rho, alpha, kwargs.get('kernel', None),
                               kwargs.get('save_undersampling', None), **kwargs)
        if self.boundary_type == 'complex_frequency_shift_PML_2' and self.kernel != 'OT2':
            raise NotImplementedError('complex_frequency_shift_PML_2 is implemented with kernel OT2')

    def _check_conditions(self, wavelets, vp, rho=None, alpha=None, preferred_kernel=None,
                          preferred_undersampling=None, **kwargs):
        """Bandwidth, dispersion and stability checks, OT2/OT4 and undersampling selection
        (devito.py:1354-1464)."""
        problem = kwargs.get('problem')
        shot_id = problem.shot.id if problem is not None else -1
        vp_ext = vp.extended_data
        vp_min, vp_max = float(np.min(vp_ext)), float(np.max(vp_ext))
        dt = self.time.step
        wav = np.atleast_2d(wavelets.data)
        f_mins, f_centres, f_maxs = [], [], []
        for w in wav:
            if np.any(w):
                a, b, c = bandwidth(w, dt, cutoff=-10)
                f_mins.append(a)
                f_centres.append(b)
                f_maxs.append(c)
        f_min = np.min(f_mins) if f_mins else 0.05 / dt
        f_max = np.max(f_maxs) if f_maxs else 0.05 / dt
        f_centre = np.median(f_centres) if f_centres else 0.05 / dt
        self._bandwidth = (f_min, f_centre, f_max)
        self._perf('(ShotID %d) Estimated bandwidth for the propagated wavelet %.3f-%.3f MHz', shot_id, f_min / 1e6,
                   f_max / 1e6)
        h = max(*self.space.spacing)
        ppw = vp_min / f_max / h if f_max > 0 else np.inf
        if ppw < 5:
            self.logger.warning('(ShotID %d) Spatial grid spacing (%.3f mm | %.3f PPW) is higher than '
                                'dispersion limit (%.3f PPW)', shot_id, h / 1e-3, ppw, 5)
        dim = self.space.dim
        dt_ot2 = (2.0 / np.pi) * h / vp_max / np.sqrt(dim)
        dt_ot4 = (3.6 / np.pi) * h / vp_max / np.sqrt(dim)
        if dt <= dt_ot2:
            selected = 'OT2'
        else:
            selected = 'OT4'
            if dt > dt_ot4:
                self.logger.warning('(ShotID %d) Time grid spacing (%.3f us) is above OT4 limit (%.3f us)',
                                    shot_id, dt / 1e-6, dt_ot4 / 1e-6)
        self.kernel = selected if preferred_kernel is None else preferred_kernel
        if self.kernel not in ('OT2', 'OT4'):
            raise ValueError('Unrecognized kernel')
        self._perf('(ShotID %d) Selected time stepping scheme %s', shot_id, self.kernel)
        dt_max = 1 / (4 * f_max)
        self.undersampling_factor = min(max(4, int(dt_max / dt)), 10) \
            if preferred_undersampling is None else int(preferred_undersampling)
        self._perf('(ShotID %d) Selected undersampling level %d', shot_id, self.undersampling_factor)

    # ---------------------------------------------------------------------------- plans

    def _density_mode(self, rho):
        if rho is None:
            return _lib.SA_DENSITY_NONE
        r = np.asarray(rho.extended_data, dtype=np.float32)
        return _lib.SA_DENSITY_CONSTANT if np.isclose(np.min(r), np.max(r)) else _lib.SA_DENSITY_VARIABLE

    def _get_plan(self, vp, rho, alpha, n_shots=1):
        space, time = self.space, self.time
        key = (space.extended_shape, space.spacing, space.extra, space.absorbing, time.step, time.extended_num,
               self.kernel, self._density_mode(rho), alpha is not None, self.undersampling_factor, n_shots,
               self.interpolation_type, self.boundary_type, float(self._bandwidth[1]), self.checkpoint_interval,
               self.checkpoint_budget)
        plan = self._plans.get(key)
        if plan is None:
            plan = _lib.Plan(space.dim, space.extended_shape, space.spacing, space.extra, space.absorbing,
                             time.step, time.extended_num, kernel=self.kernel, density=key[7],
                             attenuation=alpha is not None, undersampling=self.undersampling_factor,
                             max_shots=n_shots, interpolation=self.interpolation_type,
                             boundary='pml' if self.boundary_type == 'complex_frequency_shift_PML_2' else 'sponge',
                             f_centre=float(self._bandwidth[1]), checkpoint_interval=self.checkpoint_interval,
                             checkpoint_budget=self.checkpoint_budget)
            self._plans = {key: plan}  # one live plan: the previous one's device memory is released
        self._plan = plan
        return plan

    def _set_medium(self, plan, vp, rho, alpha):
        plan.set_medium(np.ascontiguousarray(vp.extended_data, dtype=np.float32),
                        None if rho is None else np.ascontiguousarray(rho.extended_data, dtype=np.float32),
                        None if alpha is None else np.ascontiguousarray(alpha.extended_data, dtype=np.float32))

    def _set_geometry(self, plan, shots):
        eps = (1e-3 * np.asarray(self.space.spacing)).reshape(1, -1)
        so = np.cumsum([0] + [s.num_points_sources for s in shots])
        ro = np.cumsum([0] + [s.num_points_receivers for s in shots])
        sx = np.concatenate([s.source_coordinates + eps for s in shots]).astype(np.float32)
        rx = np.concatenate([s.receiver_coordinates + eps for s in shots]).astype(np.float32)
        plan.set_geometry(so, sx, ro, rx)

    def _window(self, lo=0, hi=None):
        nt = self.time.num
        hi = self.time.extended_num if hi is None else hi
        w = scipy.signal.get_window(('tukey', 0.001), hi - lo, False)
        return np.pad(w, ((lo, nt - hi),), mode='constant', constant_values=0.)

    def _source_data(self, wavelets, diff_source):
        data = np.atleast_2d(np.asarray(wavelets.data, dtype=np.float64))
        if diff_source:  # the reference injects d/dt of the wavelet with scale 2 dt^2 vp / h
            data = np.gradient(data, self.time.step, axis=-1) * self.time.step
        return np.ascontiguousarray((data * self._window()[None, :]).astype(np.float32))

    def _save_wavefield(self, vp, rho, alpha, kwargs, wavelets=None):
        """False, 'snapshots' (p.dt2 every f steps), 'checkpoints' (both levels every K steps,
        with a checkpoint interval or budget) or 'raw' (p itself, which the reference saves when
        the wavelets, rho or alpha need a gradient, devito.py:319,410-413)."""
        raw = any(v is not None and getattr(v, 'needs_grad', False) for v in (wavelets, rho, alpha))
        save = kwargs.get('save_wavefield', False) or bool(getattr(vp, 'needs_grad', False)) or raw
        if not save:
            return False
        if raw:
            return 'raw'
        return 'checkpoints' if self.checkpoint_interval > 0 or self.checkpoint_budget > 0 else 'snapshots'

    # ---------------------------------------------------------------------------- forward

    def before_forward(self, wavelets, vp, rho=None, alpha=None, **kwargs):
        """Prepare the state run (devito.py:220-513)."""
        problem = kwargs.get('problem')
        self._check_problem(wavelets, vp, rho=rho, alpha=alpha, **kwargs)
        plan = self._get_plan(vp, rho, alpha, 1)
        self._set_medium(plan, vp, rho, alpha)
        self._set_geometry(plan, [problem.shot])
        self._src = self._source_data(wavelets, kwargs.get('diff_source', False))
        self._traces = np.zeros((plan.n_rec, self.time.extended_num), np.float32)

    def run_forward(self, wavelets, vp, rho=None, alpha=None, **kwargs):
        """Run the state loop (devito.py:515-581); empty wavelets skip the run."""
        problem = kwargs.get('problem')
        if np.linalg.norm(np.asarray(wavelets.data)) < 1e-31:
            self.logger.warning('(ShotID %d) Empty wavelets, not running forward', problem.shot.id)
            self._saved = False
            return
        save = self._save_wavefield(vp, rho, alpha, kwargs, wavelets)
        shot_id = problem.shot.id if problem is not None else -1
        points = float(np.prod(self.space.extended_shape))
        if save in ('snapshots', 'raw'):
            n_snap = (self.time.extended_num + self.undersampling_factor) // self.undersampling_factor + 1
            self._perf('(ShotID %d) Expected wavefield size %.4f GB', shot_id, n_snap * points * 4 / 1024 ** 3)
        t0 = time.perf_counter()
        self._plan.forward(self._src, self._traces, save=save)
        self._saved = save
        secs = time.perf_counter() - t0
        self._perf('(ShotID %d) Forward ran in %.3f s (%.2f GPts/s)', shot_id, secs,
                   points * (self.time.extended_num - 2) / max(secs, 1e-9) / 1e9)

    def after_forward(self, wavelets, vp, rho=None, alpha=None, **kwargs):
        """Return the modelled traces (devito.py:583-685)."""
        problem = kwargs.get('problem')
        return problem.shot.observed.alike(name='modelled', data=self._traces.copy())

    # ---------------------------------------------------------------------------- adjoint

    def before_adjoint(self, adjoint_source, wavelets, vp, rho=None, alpha=None, **kwargs):
        """Prepare the adjoint run (devito.py:689-873)."""
        if not self._saved:
            raise RuntimeError('adjoint requires a forward run that saved the wavefield (vp.needs_grad)')
        self.init_grad(wavelets, vp, rho, alpha, **kwargs)
        res = np.atleast_2d(np.asarray(adjoint_source.data, dtype=np.float64))
        self._res = np.ascontiguousarray((res * self._window()[None, :]).astype(np.float32))

    def run_adjoint(self, adjoint_source, wavelets, vp, rho=None, alpha=None, **kwargs):
        """Reverse-time adjoint and imaging condition (devito.py:875-920)."""
        problem = kwargs.get('problem')
        shape = self.space.extended_shape
        self._grad = np.zeros(shape, np.float32)
        self._prec = np.zeros(shape, np.float32)
        self._wgrad = None
        if getattr(wavelets, 'needs_grad', False):
            self._wgrad = np.zeros((self._plan.n_src, self.time.extended_num), np.float32)
        self._grad_rho = self._prec_rho = None
        if rho is not None and getattr(rho, 'needs_grad', False):
            self._grad_rho = np.zeros(shape, np.float32)
            self._prec_rho = np.zeros(shape, np.float32)
        if np.linalg.norm(np.asarray(adjoint_source.data)) < 1e-31:
            self.logger.warning('(ShotID %d) Empty adjoint source, not running adjoint', problem.shot.id)
            return
        t0 = time.perf_counter()
        self._plan.adjoint(self._res, self._grad, self._prec, grad_wavelets=self._wgrad, grad_rho=self._grad_rho,
                           prec_rho=self._prec_rho)
        secs = time.perf_counter() - t0
        steps = self.time.extended_num - 1 - self.undersampling_factor
        self._perf('(ShotID %d) Adjoint ran in %.3f s (%.2f GPts/s)', problem.shot.id if problem is not None else -1,
                   secs, float(np.prod(self.space.extended_shape)) * steps / max(secs, 1e-9) / 1e9)

    def after_adjoint(self, adjoint_source, wavelets, vp, rho=None, alpha=None, **kwargs):
        """Retrieve the gradients (devito.py:922-981)."""
        return self.get_grad(wavelets, vp, rho, alpha, **kwargs)

    # ---------------------------------------------------------------------------- gradients

    def prepare_grad_vp(self, vp, **kwargs):
        """The vp imaging condition runs as its own kernel after each adjoint step (devito.py:985-1024)."""
        return ()

    def init_grad_vp(self, vp, **kwargs):
        """Gradient buffers start at zero (devito.py:1026-1043)."""
        self._grad = None
        self._prec = None

    def get_grad_vp(self, vp, **kwargs):
        """Chain rule to slowness (default for vp, which carries the inverse transform) or to
        vp, on the inner grid, with the illumination preconditioner in ``.prec``
        (devito.py:1045-1113)."""
        inner = self.space.inner
        g = np.asarray(self._grad[inner], dtype=np.float32).copy()
        p = np.asarray(self._prec[inner], dtype=np.float32).copy()
        is_slowness = False
        if getattr(vp, 'transform', None) is not None:
            try:
                is_slowness = bool(np.isclose(1 / vp.transform(10), 10))
            except Exception:  # noqa: BLE001
                pass
        vpd = np.asarray(vp.data, dtype=np.float32)
        if is_slowness:
            g *= +1 / vpd
            p *= (1 / vpd) ** 2
        else:
            g *= -2 / vpd ** 3
            p *= (2 / vpd) ** 3 ** 2  # the reference's operator precedence (devito.py:1081)
        grad = vp.alike(name='vp_grad', data=g, shape=g.shape, extended_shape=g.shape, inner=None)
        grad.prec = vp.alike(name='vp_prec', data=p, shape=p.shape, extended_shape=p.shape, inner=None)
        return grad

    def prepare_grad_rho(self, rho, **kwargs):
        """The rho imaging condition, -grad(b, shift=-1/2) . grad(p, shift=-1/2) - b laplace(p)
        from the raw saved wavefield times p_a, runs after each adjoint step (devito.py:1115-1150)."""
        return ()

    def init_grad_rho(self, rho, **kwargs):
        """Gradient buffers start at zero (devito.py:1152-1169)."""
        self._grad_rho = None
        self._prec_rho = None

    def get_grad_rho(self, rho, **kwargs):
        """The raw rho gradient on the inner grid (no chain rule), with its preconditioner in
        ``.prec`` (devito.py:1171-1208)."""
        inner = self.space.inner
        shape = self.space.extended_shape
        gr = self._grad_rho if self._grad_rho is not None else np.zeros(shape, np.float32)
        pr = self._prec_rho if self._prec_rho is not None else np.zeros(shape, np.float32)
        g = np.asarray(gr[inner], dtype=np.float32).copy()
        p = np.asarray(pr[inner], dtype=np.float32).copy()
        grad = rho.alike(name='rho_grad', data=g, shape=g.shape, extended_shape=g.shape, inner=None)
        grad.prec = rho.alike(name='rho_prec', data=p, shape=g.shape, extended_shape=g.shape, inner=None)
        return grad

    def prepare_grad_wavelets(self, wavelets, **kwargs):
        """The wavelet gradient is gathered after each adjoint step (devito.py:755-756, 1189-1203)."""
        return ()

    def init_grad_wavelets(self, wavelets, **kwargs):
        """The gradient buffer starts at zero (devito.py:1205-1224)."""
        self._wgrad = None

    def get_grad_wavelets(self, wavelets, **kwargs):
        """-interp(p_a[t]) at the source points, [n_src, nt] (devito.py:1226-1262)."""
        g = self._wgrad if self._wgrad is not None else np.zeros(np.atleast_2d(wavelets.data).shape, np.float32)
        return wavelets.alike(name='wavelets_grad', data=g, shape=g.shape, extended_shape=g.shape, inner=None)

    # ---------------------------------------------------------------------------- batches

    def forward_batch(self, shots, vp, rho=None, alpha=None, save_wavefield=False, **kwargs):
        """Every shot of ``shots`` (uneven source/receiver counts allowed) in one plan: the
        batched form of stride.forward's per-shot loop (stride/__init__.py:117-169).
        Returns the modelled trace arrays, one [n_rec, nt] array per shot."""
        wav = shots[0].wavelets
        self._check_problem(wav, vp, rho=rho, alpha=alpha, problem=None, **kwargs)
        plan = self._get_plan(vp, rho, alpha, len(shots))
        self._set_medium(plan, vp, rho, alpha)
        self._set_geometry(plan, shots)
        src = np.concatenate([self._source_data(s.wavelets, kwargs.get('diff_source', False)) for s in shots])
        traces = np.zeros((plan.n_rec, self.time.extended_num), np.float32)
        plan.forward(src, traces, save=save_wavefield)
        self._saved = save_wavefield
        out, k = [], 0
        for s in shots:
            out.append(traces[k:k + s.num_points_receivers])
            k += s.num_points_receivers
        return out

    def gradient_batch(self, residuals, vp, rho_grad=False):
        """Adjoint of the last ``forward_batch(save_wavefield=True)``: residuals per shot,
        returns the summed raw (grad, prec) on the extended grid. ``rho_grad`` (after
        ``forward_batch(save_wavefield='raw')``): returns (grad, prec, grad_rho, prec_rho)."""
        res = np.concatenate([np.atleast_2d(r) for r in residuals]).astype(np.float64)
        res = np.ascontiguousarray((res * self._window()[None, :]).astype(np.float32))
        grad = np.zeros(self.space.extended_shape, np.float32)
        prec = np.zeros(self.space.extended_shape, np.float32)
        if rho_grad:
            gr = np.zeros(self.space.extended_shape, np.float32)
            pr = np.zeros(self.space.extended_shape, np.float32)
            self._plan.adjoint(res, grad, prec, grad_rho=gr, prec_rho=pr)
            return grad, prec, gr, pr
        self._plan.adjoint(res, grad, prec)
        return grad, prec
