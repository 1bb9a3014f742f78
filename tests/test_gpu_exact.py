"""Exact-gradient mode (SA_GRAD_EXACT): the CUDA gradient of the discrete forward map against the
FP64 exact-adjoint oracle on identical seeded inputs, and against central finite differences of
the CUDA forward itself along random directions (relative error <= 1e-2)."""

import numpy as np
import pytest

from oracle import numpy_oracle as npo
from stride_gb300 import _lib
from tests import _cases as C

pytestmark = pytest.mark.gpu


def _wavelets(c):
    wav = np.concatenate([np.tile(c['wav'][None], (len(s), 1)) for s in c['srcs']]).astype(np.float64)
    return np.ascontiguousarray((wav * C.window(c['nt'])[None, :]).astype(np.float32))


def _exact(c, plan, weights):
    tr = np.zeros((plan.n_rec, c['nt']), np.float32)
    plan.forward(_wavelets(c), tr, save='checkpoints')
    g = np.zeros(c['vp'].shape, np.float32)
    p = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(np.ascontiguousarray(weights.astype(np.float32)), g, p, exact=True)
    return tr, g


def _oracle_exact(c, weights):
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    total = np.zeros(c['vp'].shape)
    k = 0
    for s in range(len(c['srcs'])):
        nr = len(c['recs'][s])
        wav = np.tile(c['wav'][None], (len(c['srcs'][s]), 1))
        g, _ = npo.adjoint_exact(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][s], c['recs'][s],
                                 wav, weights[k:k + nr], origin, rho=c['rho'], alpha=c['alpha'], kernel=c['kernel'])
        total += g
        k += nr
    return total


@pytest.mark.parametrize('kernel,density,alpha,interval', [('OT4', 'variable', True, 16), ('OT4', 'none', False, 50),
                                                           ('OT2', 'constant', True, 7)])
def test_exact_gradient_matches_oracle(kernel, density, alpha, interval):
    c = C.small_case(kernel=kernel, density=density, alpha=alpha, inner=40, nt=180, n_shots=3, uneven=True)
    plan = C.make_plan(c, checkpoint_interval=interval)
    n_rec = sum(len(r) for r in c['recs'])
    weights = np.random.default_rng(3).standard_normal((n_rec, c['nt']))
    _, g = _exact(c, plan, weights)
    ref = _oracle_exact(c, weights)
    assert np.abs(ref).max() > 0
    assert C.cosine(g, ref) >= 0.99999
    assert C.rel_l2(g, ref) <= 2e-3


def test_exact_gradient_central_differences():
    """Misfit J = 1/2 ||traces(vp) - observed||^2 through the CUDA forward, 32 random smooth
    directions (white noise smoothed over 3 cells, peak 1 m/s per unit step). White-noise
    directions scatter strongly enough that FP32 central differences themselves carry errors of
    a few 1e-2 at useful steps."""
    scipy_ndimage = pytest.importorskip('scipy.ndimage')
    c = C.small_case(kernel='OT4', density='variable', alpha=True, inner=40, nt=220, n_shots=2)
    plan = C.make_plan(c, checkpoint_interval=20)
    true_vp = c['vp'].copy()
    obs = np.zeros((plan.n_rec, c['nt']), np.float32)
    plan.forward(_wavelets(c), obs)
    vp0 = np.where(true_vp > 0, 1500., 0.).astype(np.float32)
    plan.set_medium(vp0, c['rho'], c['alpha'])

    def misfit(vp):
        plan.set_medium(np.ascontiguousarray(vp.astype(np.float32)), c['rho'], c['alpha'])
        tr = np.zeros_like(obs)
        plan.forward(_wavelets(c), tr)
        return 0.5 * float(np.sum((tr.astype(np.float64) - obs) ** 2))

    plan.set_medium(vp0, c['rho'], c['alpha'])
    tr, g = _exact(c, plan, np.zeros_like(obs))  # forward to get the residual
    tr, g = _exact(c, plan, (tr.astype(np.float64) - obs))
    rng = np.random.default_rng(11)
    fds, ans = [], []
    for _ in range(32):
        d = scipy_ndimage.gaussian_filter(rng.standard_normal(vp0.shape), 3)
        d /= np.abs(d).max()
        eps = 1.0
        fds.append((misfit(vp0 + eps * d) - misfit(vp0 - eps * d)) / (2 * eps))
        ans.append(float(np.sum(g.astype(np.float64) * d)))
    fds, ans = np.array(fds), np.array(ans)
    # relative error over the 32 directions; per direction against the directions' RMS (a
    # direction nearly orthogonal to the gradient has a derivative at the FP32 noise level)
    assert np.linalg.norm(fds - ans) <= 1e-2 * np.linalg.norm(fds), (fds, ans)
    assert np.all(np.abs(fds - ans) <= 1e-2 * np.sqrt(np.mean(fds ** 2))), (fds, ans)


def test_exact_mode_needs_checkpoints():
    c = C.small_case(kernel='OT4', density='none', n_shots=1, nt=120)
    plan = C.make_plan(c)
    C.gpu_forward(c, plan=plan, save=True)
    with pytest.raises(_lib.StrideAccError):
        plan.adjoint(np.zeros((plan.n_rec, c['nt']), np.float32), np.zeros(c['vp'].shape, np.float32),
                     np.zeros(c['vp'].shape, np.float32), exact=True)


@pytest.mark.parametrize('interp', ['hicks', 'sinc'])
def test_exact_gradient_hicks(interp):
    """SA_GRAD_EXACT with wide-support (Hicks, sinc) sources and receivers (the forward's support in
    its transpose) against the FP64 exact-adjoint oracle with the same interpolation."""
    c = C.small_case(kernel='OT4', density='variable', alpha=True, inner=40, nt=160, n_shots=2, uneven=True)
    plan = C.make_plan(c, checkpoint_interval=16, interpolation=interp)
    n_rec = sum(len(r) for r in c['recs'])
    weights = np.random.default_rng(8).standard_normal((n_rec, c['nt']))
    _, g = _exact(c, plan, weights)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    ref = np.zeros(c['vp'].shape)
    k = 0
    for s in range(2):
        nr = len(c['recs'][s])
        wav = np.tile(c['wav'][None], (len(c['srcs'][s]), 1))
        gs, _ = npo.adjoint_exact(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][s],
                                  c['recs'][s], wav, weights[k:k + nr], origin, rho=c['rho'], alpha=c['alpha'],
                                  kernel='OT4', interpolation=interp)
        ref += gs
        k += nr
    assert np.abs(ref).max() > 0
    assert C.cosine(g, ref) >= 0.99999
    assert C.rel_l2(g, ref) <= 2e-3
