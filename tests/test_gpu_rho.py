"""The rho gradient and the raw-wavefield vp gradient (the reference's gradient path when rho or
the wavelets need a gradient, stride/physics/iso_acoustic/devito.py:410-413, 1003-1024,
1115-1150) through the C ABI against the NumPy oracle on the same seeded inputs: traces relative
L2 <= 1e-4, gradients cosine >= 0.999 and relative L2 <= 1e-3, preconditioners relative L2 <= 1e-3."""

import numpy as np
import pytest

from tests import _cases as C

pytestmark = pytest.mark.gpu


def _oracle(c, s, res, src=False):
    from oracle import numpy_oracle as npo
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    wav = np.tile(c['wav'][None], (len(c['srcs'][s]), 1))
    kw = dict(rho=c['rho'], alpha=c['alpha'], kernel='OT4', undersampling=4)
    tr, snaps = npo.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][s], c['recs'][s], wav,
                            origin, save='raw', **kw)
    out = npo.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res, origin, snaps,
                      raw=True, rho_grad=c['rho'] is not None, src_coords=c['srcs'][s] if src else None, **kw)
    return tr, out


def _residuals(c, got, seed):
    rng = np.random.default_rng(seed)
    res = [rng.standard_normal(g.shape).astype(np.float32) * np.abs(g).max() for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    return res, resw


@pytest.mark.parametrize('density', ['variable', 'constant'])
def test_rho_gradient_parity(density):
    """Three shots (one padded pair lane), uneven sources and receivers: grad/prec of vp and rho."""
    c = C.small_case(kernel='OT4', density=density, alpha=True, n_shots=3, uneven=True, nt=220, inner=48)
    plan = C.make_plan(c)
    got, plan = C.gpu_forward(c, plan=plan, save='raw')
    res, resw = _residuals(c, got, 11)
    shape = c['vp'].shape
    out = [np.zeros(shape, np.float32) for _ in range(4)]
    plan.adjoint(resw, out[0], out[1], grad_rho=out[2], prec_rho=out[3])
    ref = [np.zeros(shape) for _ in range(4)]
    for s in range(3):
        tr, o = _oracle(c, s, res[s])
        assert C.rel_l2(got[s], tr) <= 1e-4
        for k in range(4):
            ref[k] += o[k]
    for k in (0, 2):
        assert np.abs(ref[k]).max() > 0
        assert C.cosine(out[k], ref[k]) >= 0.999
        assert C.rel_l2(out[k], ref[k]) <= 1e-3
    for k in (1, 3):
        assert C.rel_l2(out[k], ref[k]) <= 1e-3
    # the vp gradient alone (sa_adjoint after the raw forward) is the same computation
    g, p = np.zeros(shape, np.float32), np.zeros(shape, np.float32)
    C.gpu_forward(c, plan=plan, save='raw')
    plan.adjoint(resw, g, p)
    assert np.array_equal(g, out[0]) and np.array_equal(p, out[1])


def test_rho_and_wavelet_gradients_together():
    """The wavelet gradient is unchanged by the raw save, and comes out with the rho gradient."""
    c = C.small_case(kernel='OT4', density='variable', alpha=False, n_shots=2, uneven=True, nt=200, inner=48)
    plan = C.make_plan(c)
    got, plan = C.gpu_forward(c, plan=plan, save='raw')
    res, resw = _residuals(c, got, 12)
    shape = c['vp'].shape
    out = [np.zeros(shape, np.float32) for _ in range(4)]
    gw = np.zeros((plan.n_src, c['nt']), np.float32)
    plan.adjoint(resw, out[0], out[1], grad_wavelets=gw, grad_rho=out[2], prec_rho=out[3])
    k = 0
    g_rho = np.zeros(shape)
    for s in range(2):
        _, o = _oracle(c, s, res[s], src=True)
        ns = len(c['srcs'][s])
        assert C.rel_l2(gw[k:k + ns], o[4]) <= 1e-4
        k += ns
        g_rho += o[2]
    assert C.cosine(out[2], g_rho) >= 0.999


def test_rho_gradient_needs_raw_forward():
    from stride_gb300 import _lib
    c = C.small_case(kernel='OT4', density='variable', n_shots=1, nt=120, inner=32)
    plan = C.make_plan(c)
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    shape = c['vp'].shape
    res = np.zeros((plan.n_rec, c['nt']), np.float32)
    with pytest.raises(_lib.StrideAccError) as e:
        plan.adjoint(res, np.zeros(shape, np.float32), np.zeros(shape, np.float32),
                     grad_rho=np.zeros(shape, np.float32), prec_rho=np.zeros(shape, np.float32))
    assert e.value.code == _lib.SA_E_INVALID
