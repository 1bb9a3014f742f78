"""The CFS-PML boundary (ComplexFrequencyShiftPML2, stride/physics/boundaries/devito.py:72-191) with
OT2 through the C ABI against the NumPy oracle on the same seeded inputs: traces relative L2
<= 1e-4, vp and rho gradients cosine >= 0.999 and relative L2 <= 1e-3."""

import numpy as np
import pytest

from tests import _cases as C

pytestmark = pytest.mark.gpu

F_CENTRE = 1.0e6  # the small case's tone burst


def _oracle(c, s, save):
    from oracle import numpy_oracle as npo
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    wav = np.tile(c['wav'][None], (len(c['srcs'][s]), 1))
    return npo.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][s], c['recs'][s], wav,
                       origin, rho=c['rho'], alpha=c['alpha'], kernel='OT2', save=save, boundary='pml',
                       f_centre=F_CENTRE)


@pytest.mark.parametrize('extra', [12, 20])
def test_pml_forward_and_gradient_parity(extra):
    """Three shots (one padded pair lane); layers of 12 and 20 cells (the two coefficient rules)."""
    from oracle import numpy_oracle as npo
    c = C.small_case(kernel='OT2', density='variable', alpha=True, n_shots=3, uneven=True, nt=260, inner=40,
                     extra=extra)
    plan = C.make_plan(c, boundary='pml', f_centre=F_CENTRE)
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    sponge, _ = C.gpu_forward(c, plan=C.make_plan(c))
    rng = np.random.default_rng(21)
    res = [rng.standard_normal(g.shape).astype(np.float32) * np.abs(g).max() for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    grad = np.zeros(c['vp'].shape, np.float32)
    prec = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(resw, grad, prec)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    g_ref = np.zeros(c['vp'].shape)
    p_ref = np.zeros(c['vp'].shape)
    for s in range(3):
        tr, snaps = _oracle(c, s, True)
        assert np.abs(tr).max() > 0
        assert C.rel_l2(got[s], tr) <= 1e-4
        assert C.rel_l2(got[s], sponge[s]) > 1e-3  # the boundary is not the sponge
        g, p = npo.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res[s], origin,
                           snaps, rho=c['rho'], alpha=c['alpha'], kernel='OT2', boundary='pml', f_centre=F_CENTRE)
        g_ref += g
        p_ref += p
    assert C.cosine(grad, g_ref) >= 0.999
    assert C.rel_l2(grad, g_ref) <= 1e-3
    assert C.rel_l2(prec, p_ref) <= 1e-3


def test_pml_rho_gradient_parity():
    """Raw save and the rho gradient with the CFS-PML."""
    from oracle import numpy_oracle as npo
    c = C.small_case(kernel='OT2', density='variable', alpha=False, n_shots=2, nt=240, inner=40)
    plan = C.make_plan(c, boundary='pml', f_centre=F_CENTRE)
    got, plan = C.gpu_forward(c, plan=plan, save='raw')
    rng = np.random.default_rng(22)
    res = [rng.standard_normal(g.shape).astype(np.float32) * np.abs(g).max() for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    shape = c['vp'].shape
    out = [np.zeros(shape, np.float32) for _ in range(4)]
    plan.adjoint(resw, out[0], out[1], grad_rho=out[2], prec_rho=out[3])
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    ref = [np.zeros(shape) for _ in range(4)]
    for s in range(2):
        tr, raw = _oracle(c, s, 'raw')
        assert C.rel_l2(got[s], tr) <= 1e-4
        o = npo.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res[s], origin, raw,
                        rho=c['rho'], kernel='OT2', raw=True, rho_grad=True, boundary='pml', f_centre=F_CENTRE)
        for k in range(4):
            ref[k] += o[k]
    for k in (0, 2):
        assert C.cosine(out[k], ref[k]) >= 0.999
        assert C.rel_l2(out[k], ref[k]) <= 1e-3


def test_pml_plan_limits():
    from stride_gb300 import _lib
    c = C.small_case(kernel='OT4', n_shots=1, nt=60, inner=32)
    with pytest.raises(_lib.StrideAccError) as e:
        C.make_plan(c, boundary='pml', f_centre=F_CENTRE)
    assert e.value.code == _lib.SA_E_UNSUPPORTED
    c = C.small_case(kernel='OT2', n_shots=1, nt=60, inner=32)
    plan = C.make_plan(c, boundary='pml', f_centre=F_CENTRE)
    C.gpu_forward(c, plan=plan, save='checkpoints')
    shape = c['vp'].shape
    res = np.zeros((plan.n_rec, c['nt']), np.float32)
    with pytest.raises(_lib.StrideAccError) as e:  # the exact adjoint holds no CFS-PML terms
        plan.adjoint(res, np.zeros(shape, np.float32), np.zeros(shape, np.float32), exact=True)
    assert e.value.code == _lib.SA_E_UNSUPPORTED
