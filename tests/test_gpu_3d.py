"""3D parity of the CUDA path (through the C ABI) with the C oracle on identical seeded inputs:
traces relative L2 <= 1e-4, parity-mode vp gradient cosine >= 0.999 and relative L2 <= 1e-3."""

import numpy as np
import pytest

from oracle import c_oracle
from oracle import numpy_oracle as npo
from stride_gb300 import _lib, phantoms
from tests import _cases as C

pytestmark = pytest.mark.gpu


def case3d(kernel='OT4', density='variable', alpha=True, inner=24, nt=160, seed=2, n_shots=1):
    rng = np.random.default_rng(seed)
    e = 8
    h = 0.5e-3
    shape_i = (inner, inner + 2, inner + 5)
    vpi, rhoi, ali = phantoms.ellipse_phantom(shape_i, (h, h, h), 3, rng, rho_range=(950., 1100.),
                                              alpha_range=(0., 1.), disk_radius=3e-3, axes=(1.5e-3, 4e-3))
    ext = (e, e, e)
    vp = phantoms.extend(vpi, ext)
    rho = None
    if density == 'variable':
        rho = phantoms.extend(rhoi, ext)
    elif density == 'constant':
        rho = np.full(vp.shape, 1000., np.float32)
    al = phantoms.extend(ali, ext) if alpha else None
    dt = (0.6 if kernel == 'OT4' else 0.35) * h / 1650.
    c = np.array([(s - 1) * h / 2 for s in shape_i])
    pts = c + 0.35 * (inner - 1) * h * np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [-1, 0, 0], [0, -1, 0.3],
                                                  [0.5, 0.5, -0.6], [-0.6, 0.4, 0.2]])
    wav = npo.tone_burst(1.0e6, 3, nt, dt)
    srcs = [pts[[s % len(pts)]] for s in range(n_shots)]
    recs = [pts for _ in range(n_shots)]
    return dict(vp=vp, rho=rho, alpha=al, spacing=(h, h, h), dt=dt, nt=nt, extra=ext, absorbing=ext, kernel=kernel,
                srcs=srcs, recs=recs, wav=wav)


def make_plan3(c, **plan_kw):
    plan = _lib.Plan(3, c['vp'].shape, c['spacing'], c['extra'], c['absorbing'], c['dt'], c['nt'], kernel=c['kernel'],
                     density=C.density_mode(c['rho']), attenuation=c['alpha'] is not None, undersampling=4,
                     max_shots=len(c['srcs']), **plan_kw)
    plan.set_medium(np.ascontiguousarray(c['vp']), None if c['rho'] is None else np.ascontiguousarray(c['rho']),
                    None if c['alpha'] is None else np.ascontiguousarray(c['alpha']))
    eps = 1e-3 * np.asarray(c['spacing'])
    so = np.cumsum([0] + [len(s) for s in c['srcs']])
    ro = np.cumsum([0] + [len(r) for r in c['recs']])
    sx = np.concatenate([np.asarray(s, np.float32) + eps for s in c['srcs']]).astype(np.float32)
    rx = np.concatenate([np.asarray(r, np.float32) + eps for r in c['recs']]).astype(np.float32)
    plan.set_geometry(so, sx, ro, rx)
    return plan


def oracle3(c, shot, save=False):
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    return c_oracle.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][shot], c['recs'][shot],
                            np.tile(c['wav'][None], (len(c['srcs'][shot]), 1)), origin, rho=c['rho'],
                            alpha=c['alpha'], kernel=c['kernel'], save=save, undersampling=4)


@pytest.mark.parametrize('kernel', ['OT2', 'OT4'])
@pytest.mark.parametrize('density,alpha', [('none', False), ('variable', True), ('constant', True)])
def test_forward_3d(kernel, density, alpha):
    c = case3d(kernel=kernel, density=density, alpha=alpha)
    got, _ = C.gpu_forward(c, plan=make_plan3(c))
    ref, _ = oracle3(c, 0)
    assert np.abs(ref).max() > 0
    assert C.rel_l2(got[0], ref) <= 1e-4


def test_gradient_3d_two_shots():
    c = case3d(kernel='OT4', density='variable', alpha=True, n_shots=2)
    plan = make_plan3(c)
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    res = [g * np.float32(0.8) for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    grad = np.zeros(c['vp'].shape, np.float32)
    prec = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(resw, grad, prec)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    g_ref = np.zeros(c['vp'].shape)
    p_ref = np.zeros(c['vp'].shape)
    for s in range(2):
        _, snaps = oracle3(c, s, save=True)
        g, p = c_oracle.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res[s], origin,
                                snaps, rho=c['rho'], alpha=c['alpha'], kernel='OT4', undersampling=4)
        g_ref += g
        p_ref += p
    assert C.cosine(grad, g_ref) >= 0.999
    assert C.rel_l2(grad, g_ref) <= 1e-3
    assert C.rel_l2(prec, p_ref) <= 1e-4


@pytest.mark.parametrize('density', ['variable', 'constant'])
def test_rho_gradient_3d_two_shots(density):
    """Raw save and the rho gradient in 3D (the raw-wavefield path of iso_acoustic/devito.py:410-413,
    1003-1024, 1115-1150) against the NumPy oracle: traces relative L2 <= 1e-4, vp and rho gradients
    cosine >= 0.999 and relative L2 <= 1e-3."""
    c = case3d(kernel='OT4', density=density, alpha=True, n_shots=2, nt=140)
    plan = make_plan3(c)
    got, plan = C.gpu_forward(c, plan=plan, save='raw')
    res = [g * np.float32(0.8) for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    shape = c['vp'].shape
    out = [np.zeros(shape, np.float32) for _ in range(4)]
    plan.adjoint(resw, out[0], out[1], grad_rho=out[2], prec_rho=out[3])
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    ref = [np.zeros(shape) for _ in range(4)]
    kw = dict(rho=c['rho'], alpha=c['alpha'], kernel='OT4', undersampling=4)
    for s in range(2):
        wav = np.tile(c['wav'][None], (len(c['srcs'][s]), 1))
        tr, raw = npo.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][s], c['recs'][s],
                              wav, origin, save='raw', **kw)
        assert C.rel_l2(got[s], tr) <= 1e-4
        o = npo.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res[s], origin, raw,
                        raw=True, rho_grad=True, **kw)
        for k in range(4):
            ref[k] += o[k]
    for k in (0, 2):
        assert np.abs(ref[k]).max() > 0
        assert C.cosine(out[k], ref[k]) >= 0.999
        assert C.rel_l2(out[k], ref[k]) <= 1e-3
    for k in (1, 3):
        assert C.rel_l2(out[k], ref[k]) <= 1e-3


def test_wavelet_gradient_3d():
    """-interp(p_a[t]) at the sources in 3D (src.interpolate(expr=-p_a), iso_acoustic/devito.py:755-756)
    against the NumPy oracle; the checkpointed adjoint gives the same values bitwise."""
    c = case3d(kernel='OT4', density='variable', alpha=True, n_shots=2, nt=120)
    plan = make_plan3(c)
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    res = [g * np.float32(0.8) for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    shape = c['vp'].shape
    gw = np.zeros((plan.n_src, c['nt']), np.float32)
    plan.adjoint(resw, np.zeros(shape, np.float32), np.zeros(shape, np.float32), grad_wavelets=gw)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    k = 0
    for s in range(2):
        _, snaps = oracle3(c, s, save=True)
        _, _, g_ref = npo.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res[s],
                                  origin, snaps, rho=c['rho'], alpha=c['alpha'], kernel='OT4', undersampling=4,
                                  src_coords=c['srcs'][s])
        ns = len(c['srcs'][s])
        assert np.abs(g_ref).max() > 0
        assert C.rel_l2(gw[k:k + ns], g_ref) <= 1e-4
        k += ns
    ck = make_plan3(c, checkpoint_interval=20)
    C.gpu_forward(c, plan=ck, save='checkpoints')
    gw2 = np.zeros_like(gw)
    ck.adjoint(resw, np.zeros(shape, np.float32), np.zeros(shape, np.float32), grad_wavelets=gw2)
    assert np.array_equal(gw, gw2)


@pytest.mark.parametrize('kernel,density,alpha,interval', [('OT4', 'variable', True, 16), ('OT2', 'constant', False, 12)])
def test_exact_gradient_3d(kernel, density, alpha, interval):
    """SA_GRAD_EXACT on a 3D plan (checkpoints, segment recompute) against the FP64 exact-adjoint
    oracle, and through torch.autograd (WaveOperator) the same gradient."""
    import torch
    from stride_gb300.autograd import WaveOperator
    c = case3d(kernel=kernel, density=density, alpha=alpha, inner=16, nt=90, n_shots=2)
    plan = make_plan3(c, checkpoint_interval=interval)
    C.gpu_forward(c, plan=plan, save='checkpoints')
    n_rec = sum(len(r) for r in c['recs'])
    weights = np.random.default_rng(5).standard_normal((n_rec, c['nt']))
    g = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(np.ascontiguousarray(weights.astype(np.float32)), g, np.zeros_like(g), exact=True)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    ref = np.zeros(c['vp'].shape)
    k = 0
    for s in range(2):
        nr = len(c['recs'][s])
        wav = np.tile(c['wav'][None], (len(c['srcs'][s]), 1))
        gs, _ = npo.adjoint_exact(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][s],
                                  c['recs'][s], wav, weights[k:k + nr], origin, rho=c['rho'], alpha=c['alpha'],
                                  kernel=kernel)
        ref += gs
        k += nr
    assert np.abs(ref).max() > 0
    assert C.cosine(g, ref) >= 0.9999
    assert C.rel_l2(g, ref) <= 2e-3
    # the same gradient through torch.autograd
    so = np.cumsum([0] + [len(x) for x in c['srcs']])
    ro = np.cumsum([0] + [len(x) for x in c['recs']])
    eps = 1e-3 * np.asarray(c['spacing'])
    sx = (np.concatenate(c['srcs']) + eps).astype(np.float32)
    rx = (np.concatenate(c['recs']) + eps).astype(np.float32)
    wav = np.concatenate([np.tile(c['wav'][None], (len(x), 1)) for x in c['srcs']]).astype(np.float64)
    wav = (wav * C.window(c['nt'])[None, :]).astype(np.float32)
    op = WaveOperator(c['vp'].shape, c['spacing'], c['extra'], c['absorbing'], c['dt'], c['nt'], so, sx, ro, rx, wav,
                      rho=c['rho'], alpha=c['alpha'], kernel=kernel, checkpoint_interval=interval)
    vp = torch.tensor(c['vp'], device='cuda', requires_grad=True)
    w = torch.tensor(weights.astype(np.float32), device='cuda')
    (op(vp) * w).sum().backward()
    assert C.rel_l2(vp.grad.cpu().numpy(), g) <= 1e-5
    op.close()


@pytest.mark.parametrize('density,interp', [('none', 'hicks'), ('variable', 'hicks'), ('variable', 'sinc')])
def test_hicks_3d(density, interp):
    """Wide-support sources and receivers on a 3D plan (Hicks, common/devito.py:640-648,843-885;
    sinc, :634-638): traces and the vp gradient against the NumPy oracle with the same
    interpolation."""
    c = case3d(kernel='OT4', density=density, alpha=True, n_shots=2, nt=120)
    plan = make_plan3(c, interpolation=interp)
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    kw = dict(rho=c['rho'], alpha=c['alpha'], kernel='OT4', interpolation=interp)
    snaps = []
    for s in range(2):
        wav = np.tile(c['wav'][None], (len(c['srcs'][s]), 1))
        ref, sn = npo.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][s], c['recs'][s],
                              wav, origin, save=True, **kw)
        assert np.abs(ref).max() > 0
        assert C.rel_l2(got[s], ref) <= 1e-4
        snaps.append(sn)
    lin, _ = C.gpu_forward(c, plan=make_plan3(c))
    assert C.rel_l2(got[0], lin[0]) > 1e-3  # the interpolation is not the linear one
    res = [g * np.float32(0.8) for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    grad = np.zeros(c['vp'].shape, np.float32)
    prec = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(resw, grad, prec)
    g_ref = np.zeros(c['vp'].shape)
    for s in range(2):
        g, _ = npo.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res[s], origin,
                           snaps[s], **kw)
        g_ref += g
    assert C.cosine(grad, g_ref) >= 0.999
    assert C.rel_l2(grad, g_ref) <= 1e-3


def test_cfs_pml_3d():
    """The CFS-PML (OT2) on a 3D plan: traces and the vp gradient against the NumPy restatement
    (ComplexFrequencyShiftPML2, stride/physics/boundaries/devito.py:72-191)."""
    c = case3d(kernel='OT2', density='variable', alpha=True, n_shots=2, nt=140)
    plan = make_plan3(c, boundary='pml', f_centre=1.0e6)
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    sponge, _ = C.gpu_forward(c, plan=make_plan3(c))
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    kw = dict(rho=c['rho'], alpha=c['alpha'], kernel='OT2', boundary='pml', f_centre=1.0e6)
    snaps = []
    for s in range(2):
        wav = np.tile(c['wav'][None], (len(c['srcs'][s]), 1))
        ref, sn = npo.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][s], c['recs'][s],
                              wav, origin, save=True, **kw)
        assert np.abs(ref).max() > 0
        assert C.rel_l2(got[s], ref) <= 1e-4
        assert C.rel_l2(got[s], sponge[s]) > 1e-3
        snaps.append(sn)
    res = [g * np.float32(0.8) for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    grad = np.zeros(c['vp'].shape, np.float32)
    prec = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(resw, grad, prec)
    g_ref = np.zeros(c['vp'].shape)
    for s in range(2):
        g, _ = npo.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res[s], origin,
                           snaps[s], **kw)
        g_ref += g
    assert C.cosine(grad, g_ref) >= 0.999
    assert C.rel_l2(grad, g_ref) <= 1e-3


def test_wavelet_gradient_hicks_3d():
    """The wavelet gradient with Hicks interpolation on a 3D plan against the NumPy oracle."""
    c = case3d(kernel='OT4', density='variable', alpha=False, n_shots=2, nt=110)
    plan = make_plan3(c, interpolation='hicks')
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    res = [g * np.float32(0.8) for g in got]
    resw = np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :]).astype(np.float32))
    shape = c['vp'].shape
    gw = np.zeros((plan.n_src, c['nt']), np.float32)
    plan.adjoint(resw, np.zeros(shape, np.float32), np.zeros(shape, np.float32), grad_wavelets=gw)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    kw = dict(rho=c['rho'], alpha=c['alpha'], kernel='OT4', interpolation='hicks')
    k = 0
    for s in range(2):
        wav = np.tile(c['wav'][None], (len(c['srcs'][s]), 1))
        _, snaps = npo.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][s], c['recs'][s],
                               wav, origin, save=True, **kw)
        _, _, g_ref = npo.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][s], res[s],
                                  origin, snaps, src_coords=c['srcs'][s], **kw)
        ns = len(c['srcs'][s])
        assert np.abs(g_ref).max() > 0
        assert C.rel_l2(gw[k:k + ns], g_ref) <= 1e-4
        k += ns


@pytest.mark.parametrize('interp', ['hicks', 'sinc'])
def test_exact_gradient_hicks_3d(interp):
    """SA_GRAD_EXACT on a 3D plan with a wide support (Hicks, sinc) against the FP64 exact-adjoint
    oracle."""
    c = case3d(kernel='OT4', density='variable', alpha=True, inner=20, nt=80, n_shots=2)
    plan = make_plan3(c, checkpoint_interval=16, interpolation=interp)
    C.gpu_forward(c, plan=plan, save='checkpoints')
    n_rec = sum(len(r) for r in c['recs'])
    weights = np.random.default_rng(7).standard_normal((n_rec, c['nt']))
    g = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(np.ascontiguousarray(weights.astype(np.float32)), g, np.zeros_like(g), exact=True)
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
    assert C.cosine(g, ref) >= 0.9999
    assert C.rel_l2(g, ref) <= 2e-3


def test_autotune_3d_layout_and_cache():
    """sa_autotune on a 3D plan picks a tile and x chunking by timing them; every point's arithmetic
    is the same in any layout, so the traces are bitwise unchanged, and a second plan of the same
    shape takes the cached layout."""
    c = case3d(kernel='OT4', density='variable', alpha=True, n_shots=3, nt=60)
    plan = make_plan3(c)
    before, _ = C.gpu_forward(c, plan=plan)
    plan.autotune()
    tuned = plan.layout
    after, _ = C.gpu_forward(c, plan=plan)
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    twin = make_plan3(c)
    C.gpu_forward(c, plan=twin)
    twin.autotune()
    assert twin.layout == tuned
    C.gpu_forward(c, plan=twin, save=True)
    with pytest.raises(_lib.StrideAccError) as e:  # the saved wavefield would be overwritten
        twin.autotune()
    assert e.value.code == _lib.SA_E_INVALID



def test_odd_batch_pairs_and_lone_shot_are_bitwise_equal():
    """An odd batch runs its shot pairs in the two-lane kernel and its last shot in the one-lane form;
    every lane's arithmetic is the same, so each shot's traces equal those of a one-shot plan bit for
    bit, and the batch matches the oracle."""
    c = case3d(kernel='OT4', density='variable', alpha=True, n_shots=3, nt=80)
    batch, _ = C.gpu_forward(c, plan=make_plan3(c))
    for s in range(3):
        one = dict(c, srcs=[c['srcs'][s]], recs=[c['recs'][s]])
        alone, _ = C.gpu_forward(one, plan=make_plan3(one))
        assert np.array_equal(batch[s], alone[0])
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    wav = np.tile(c['wav'][None], (len(c['srcs'][2]), 1))
    ref, _ = npo.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][2], c['recs'][2], wav,
                         origin, rho=c['rho'], alpha=c['alpha'], kernel='OT4')
    assert C.rel_l2(batch[2], ref) <= 1e-4
