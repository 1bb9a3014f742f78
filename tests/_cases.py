"""Shared case builders for the parity tests: run the same seeded inputs through the CUDA
path (C ABI) and the C oracle."""

import numpy as np

from oracle import c_oracle
from oracle import numpy_oracle as npo
from stride_gb300 import phantoms


def small_case(kernel='OT4', density='none', alpha=False, inner=64, nt=300, seed=0, n_shots=1, uneven=False, extra=12):
    """A reduced 2D case with the structure of the benchmark workloads."""
    rng = np.random.default_rng(seed)
    h = 0.5e-3
    shape_i = (inner, inner + 7)  # non-square on purpose
    vpi, rhoi, ali = phantoms.ellipse_phantom(shape_i, (h, h), 4, rng, rho_range=(950., 1100.),
                                              alpha_range=(0., 1.), disk_radius=8e-3, axes=(2e-3, 6e-3))
    ext = (extra, extra)
    vp = phantoms.extend(vpi, ext)
    rho = None
    if density == 'variable':
        rho = phantoms.extend(rhoi, ext)
    elif density == 'constant':
        rho = np.full(vp.shape, 1000., np.float32)
    al = phantoms.extend(ali, ext) if alpha else None
    cfl = 0.6 if kernel == 'OT4' else 0.4
    dt = cfl * h / 1650.
    centre = ((shape_i[0] - 1) * h / 2, (shape_i[1] - 1) * h / 2)
    geo = phantoms.circle_geometry(24, 0.4 * (inner - 1) * h, centre, jitter=0.5, spacing=(h, h), rng=rng)
    wav = npo.tone_burst(1.0e6, 3, nt, dt)
    srcs, recs = [], []
    for s in range(n_shots):
        ns = 1 + (s % 2 if uneven else 0)
        nr = 24 - (3 * s if uneven else 0)
        srcs.append(geo[[(2 * s + k) % 24 for k in range(ns)]])
        recs.append(geo[:max(nr, 1)])
    return dict(vp=vp, rho=rho, alpha=al, spacing=(h, h), dt=dt, nt=nt, extra=ext, absorbing=ext,
                kernel=kernel, srcs=srcs, recs=recs, wav=wav, vp_inner=vpi)


def density_mode(rho):
    from stride_gb300 import _lib
    if rho is None:
        return _lib.SA_DENSITY_NONE
    r = rho.astype(np.float32)
    return _lib.SA_DENSITY_CONSTANT if np.isclose(np.min(r), np.max(r)) else _lib.SA_DENSITY_VARIABLE


def window(nt):
    return npo.tukey(nt)


def make_plan(c, max_shots=None, **plan_kw):
    from stride_gb300 import _lib
    n_shots = len(c['srcs'])
    plan = _lib.Plan(2, c['vp'].shape, c['spacing'], c['extra'], c['absorbing'], c['dt'], c['nt'],
                     kernel=c['kernel'], density=density_mode(c['rho']), attenuation=c['alpha'] is not None,
                     undersampling=4, max_shots=max_shots or n_shots, **plan_kw)
    plan.set_medium(np.ascontiguousarray(c['vp']),
                    None if c['rho'] is None else np.ascontiguousarray(c['rho']),
                    None if c['alpha'] is None else np.ascontiguousarray(c['alpha']))
    eps = 1e-3 * np.asarray(c['spacing'])
    so = np.cumsum([0] + [len(s) for s in c['srcs']])
    ro = np.cumsum([0] + [len(r) for r in c['recs']])
    sx = np.concatenate([np.asarray(s, np.float32) + eps for s in c['srcs']]).astype(np.float32)
    rx = np.concatenate([np.asarray(r, np.float32) + eps for r in c['recs']]).astype(np.float32)
    plan.set_geometry(so, sx, ro, rx)
    return plan


def gpu_forward(c, plan=None, save=False):
    """Traces per shot from the CUDA path (host buffers through the C ABI)."""
    plan = plan or make_plan(c)
    nt = c['nt']
    wav = np.concatenate([np.tile(c['wav'][None], (len(s), 1)) for s in c['srcs']]).astype(np.float64)
    wav = np.ascontiguousarray((wav * window(nt)[None, :]).astype(np.float32))
    tr = np.zeros((plan.n_rec, nt), np.float32)
    plan.forward(wav, tr, save=save)
    out, k = [], 0
    for r in c['recs']:
        out.append(tr[k:k + len(r)])
        k += len(r)
    return out, plan


def oracle_forward(c, shot, save=False):
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    wav = np.tile(c['wav'][None], (len(c['srcs'][shot]), 1))
    return c_oracle.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][shot],
                            c['recs'][shot], wav, origin, rho=c['rho'], alpha=c['alpha'], kernel=c['kernel'],
                            save=save, undersampling=4)


def oracle_adjoint(c, shot, residual, snaps):
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    return c_oracle.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][shot], residual,
                            origin, snaps, rho=c['rho'], alpha=c['alpha'], kernel=c['kernel'], undersampling=4)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def cosine(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b)))
