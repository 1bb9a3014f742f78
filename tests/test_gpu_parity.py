"""Parity of the CUDA path (through the C ABI) with the C oracle on identical seeded inputs.

Tolerances (FP32 throughout): traces relative L2 <= 1e-4; the parity-mode vp gradient
(the reference's imaging condition) relative L2 <= 1e-3 and cosine >= 0.999.
"""

import numpy as np
import pytest

from tests import _cases as C

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-4


@pytest.mark.parametrize('kernel', ['OT2', 'OT4'])
@pytest.mark.parametrize('density', ['none', 'variable', 'constant'])
@pytest.mark.parametrize('alpha', [False, True])
def test_forward_variants(kernel, density, alpha):
    c = C.small_case(kernel=kernel, density=density, alpha=alpha)
    got, _ = C.gpu_forward(c)
    ref, _ = C.oracle_forward(c, 0)
    assert np.abs(ref).max() > 0
    err = C.rel_l2(got[0], ref)
    assert err <= TRACE_TOL, err
    # rows 0 and nt-1 stay zero as in the reference's time_m=1, time_M=nt-2 loop
    assert np.all(got[0][:, 0] == 0) and np.all(got[0][:, -1] == 0)


def test_batched_uneven_shots():
    c = C.small_case(kernel='OT4', density='variable', alpha=True, n_shots=5, uneven=True)
    got, _ = C.gpu_forward(c)
    for s in range(5):
        ref, _ = C.oracle_forward(c, s)
        assert C.rel_l2(got[s], ref) <= TRACE_TOL, s


def test_single_shot_full_size():
    """The single-shot workload (256^2 inner at 0.5 mm, 2000 steps, 128 receivers)."""
    from stride_gb300 import phantoms
    w = phantoms.workload('single')
    c = dict(vp=w['vp'], rho=None, alpha=None, spacing=w['spacing'], dt=w['dt'], nt=w['nt'], extra=w['extra'],
             absorbing=w['absorbing'], kernel='OT4', srcs=w['src'], recs=w['rec'], wav=w['wavelet'])
    got, _ = C.gpu_forward(c)
    ref, _ = C.oracle_forward(c, 0)
    assert C.rel_l2(got[0], ref) <= TRACE_TOL


@pytest.mark.parametrize('density,alpha', [('none', False), ('variable', True), ('constant', False)])
def test_adjoint_gradient_parity(density, alpha):
    c = C.small_case(kernel='OT4', density=density, alpha=alpha, n_shots=2)
    plan = C.make_plan(c)
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    rng = np.random.default_rng(1)
    res = [rng.standard_normal(g.shape).astype(np.float32) * np.abs(g).max() for g in got]
    resw = np.ascontiguousarray(np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32)
    N = c['vp'].size
    grad = np.zeros(c['vp'].shape, np.float32)
    prec = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(resw, grad, prec)
    g_ref = np.zeros(c['vp'].shape, np.float64)
    p_ref = np.zeros(c['vp'].shape, np.float64)
    for s in range(2):
        _, snaps = C.oracle_forward(c, s, save=True)
        g, p = C.oracle_adjoint(c, s, res[s], snaps)
        g_ref += g
        p_ref += p
    assert N == grad.size
    assert C.cosine(grad, g_ref) >= 0.999
    assert C.rel_l2(grad, g_ref) <= 1e-3
    assert C.rel_l2(prec, p_ref) <= 1e-4


def test_wavelet_gradient_parity():
    """-interp(p_a[t]) at the sources (src.interpolate(expr=-p_a)) for two shots, uneven sources."""
    from oracle import numpy_oracle as npo
    c = C.small_case(kernel='OT4', density='variable', alpha=True, n_shots=2, uneven=True, nt=220)
    plan = C.make_plan(c)
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    rng = np.random.default_rng(4)
    res = [rng.standard_normal(g.shape).astype(np.float32) * np.abs(g).max() for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    grad = np.zeros(c['vp'].shape, np.float32)
    prec = np.zeros(c['vp'].shape, np.float32)
    gw = np.zeros((plan.n_src, c['nt']), np.float32)
    plan.adjoint(resw, grad, prec, grad_wavelets=gw)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    k = 0
    for s in range(2):
        _, snaps = C.oracle_forward(c, s, save=True)
        _, _, g_ref = npo.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res[s], origin,
                                  snaps, rho=c['rho'], alpha=c['alpha'], kernel='OT4', undersampling=4,
                                  src_coords=c['srcs'][s])
        ns = len(c['srcs'][s])
        assert np.abs(g_ref).max() > 0
        assert C.rel_l2(gw[k:k + ns], g_ref) <= 1e-4
        k += ns
    # the vp gradient is unchanged by the extra outputs
    g2 = np.zeros_like(grad)
    C.gpu_forward(c, plan=plan, save=True)
    plan.adjoint(resw, g2, np.zeros_like(prec))
    assert np.array_equal(grad, g2)


@pytest.mark.parametrize('interp', ['hicks', 'sinc'])
@pytest.mark.parametrize('density', ['none', 'variable'])
def test_hicks_interpolation_parity(density, interp):
    """Wide-support sources and receivers (Hicks: 8 points per axis, the sources smoothed; sinc:
    Devito's half-width 7): traces and the vp gradient against the NumPy oracle with the same
    interpolation."""
    from oracle import numpy_oracle as npo
    c = C.small_case(kernel='OT4', density=density, alpha=True, n_shots=2, uneven=True, nt=200, inner=48)
    plan = C.make_plan(c, interpolation=interp)
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    snaps_all = []
    for s in range(2):
        wav = np.tile(c['wav'][None], (len(c['srcs'][s]), 1))
        ref, snaps = npo.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][s], c['recs'][s],
                                 wav, origin, rho=c['rho'], alpha=c['alpha'], kernel='OT4', save=True,
                                 interpolation=interp)
        assert np.abs(ref).max() > 0
        assert C.rel_l2(got[s], ref) <= 1e-4
        snaps_all.append(snaps)
    rng = np.random.default_rng(8)
    res = [rng.standard_normal(g.shape).astype(np.float32) * np.abs(g).max() for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    grad = np.zeros(c['vp'].shape, np.float32)
    prec = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(resw, grad, prec)
    g_ref = np.zeros(c['vp'].shape)
    for s in range(2):
        g, _ = npo.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res[s], origin,
                           snaps_all[s], rho=c['rho'], alpha=c['alpha'], kernel='OT4', interpolation=interp)
        g_ref += g
    assert C.cosine(grad, g_ref) >= 0.999
    assert C.rel_l2(grad, g_ref) <= 1e-3


@pytest.mark.parametrize('interp', ['hicks', 'sinc'])
def test_wavelet_gradient_hicks(interp):
    """The wavelet gradient with a wide support: -interp(p_a) over the sources' support (Hicks:
    smoothed, 8 x 8; sinc: 14 x 14), against the NumPy oracle."""
    from oracle import numpy_oracle as npo
    c = C.small_case(kernel='OT4', density='variable', alpha=True, n_shots=2, uneven=True, nt=200, inner=48)
    plan = C.make_plan(c, interpolation=interp)
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    rng = np.random.default_rng(6)
    res = [rng.standard_normal(g.shape).astype(np.float32) * np.abs(g).max() for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    gw = np.zeros((plan.n_src, c['nt']), np.float32)
    plan.adjoint(resw, np.zeros(c['vp'].shape, np.float32), np.zeros(c['vp'].shape, np.float32), grad_wavelets=gw)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    k = 0
    for s in range(2):
        wav = np.tile(c['wav'][None], (len(c['srcs'][s]), 1))
        _, snaps = npo.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][s], c['recs'][s],
                               wav, origin, rho=c['rho'], alpha=c['alpha'], kernel='OT4', save=True,
                               interpolation=interp)
        _, _, g_ref = npo.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res[s], origin,
                                  snaps, rho=c['rho'], alpha=c['alpha'], kernel='OT4', interpolation=interp,
                                  src_coords=c['srcs'][s])
        ns = len(c['srcs'][s])
        assert np.abs(g_ref).max() > 0
        assert C.rel_l2(gw[k:k + ns], g_ref) <= 1e-4
        k += ns
