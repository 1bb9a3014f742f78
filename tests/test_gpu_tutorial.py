"""The CUDA path against values the reference itself computed: all 15 per-shot losses of the first
FWI iteration recorded in the reference's imaging tutorial (breast2D true model, 456 x 485 extended
grid with a 40-cell sponge inside 50 extra cells, 2500 OT2 steps; tests/_tutorial.py), with the 15
shots batched in one plan, and the traces of one shot against the C oracle."""

import numpy as np
import pytest

from oracle import c_oracle
from tests import _cases as C
from tests import _tutorial as T

pytestmark = pytest.mark.gpu


def test_cuda_path_reproduces_the_recorded_tutorial_losses():
    g = T.load()
    shots = g['shot_ids'].tolist()
    w = T.wavelet(g)
    obs_case = T.case(g, g['vp_true'], w, shots)
    mod_case = T.case(g, np.full(g['vp_true'].shape, 1500., np.float32),
                      T.process_wavelet(w, T.PERIOD_RECORDED), shots)
    obs, _ = C.gpu_forward(obs_case)
    mod, _ = C.gpu_forward(mod_case)
    for k, s in enumerate(shots):
        got = T.loss(obs[k], mod[k], T.PERIOD_RECORDED)
        assert abs(got - g['losses'][k]) <= 3e-3 * g['losses'][k], (s, got, g['losses'][k])
    origin = tuple(-e * h for e, h in zip(obs_case['extra'], obs_case['spacing']))
    ref, _ = c_oracle.forward(obs_case['vp'], obs_case['spacing'], obs_case['dt'], obs_case['nt'],
                              obs_case['absorbing'], obs_case['srcs'][0], obs_case['recs'][0], w[None], origin,
                              kernel='OT2')
    assert C.rel_l2(obs[0], ref) <= 1e-4


def test_product_pipelines_reproduce_the_recorded_total_loss():
    """The same first iteration through the product's own GPU trace pipelines and FWI driver
    (fwi.PlainFWI.misfit: filters, mute, norm per shot, L2 on the device) against the tutorial's
    recorded total over the 15 shots (26.2682). The filters' cosine tables depend only on their
    period: f_max 0.42 MHz at relaxation 1 gives the recorded run's 31-tap table (1 / f = 14.88)."""
    import torch
    from stride_gb300 import fwi

    g = T.load()
    shots = g['shot_ids'].tolist()
    c = T.case(g, g['vp_true'], T.wavelet(g), shots)
    w = dict(shape=c['vp'].shape, spacing=c['spacing'], extra=c['extra'], absorbing=c['absorbing'], dt=c['dt'],
             nt=c['nt'], vp=c['vp'], rho=None, alpha=None, shots=shots, src=c['srcs'], rec=c['recs'],
             wavelet=c['wav'].astype(np.float32))
    plain = fwi.PlainFWI(w, kernel='OT2')
    try:
        total = plain.misfit(torch.full(c['vp'].shape, 1500., device=plain.device), f_max=0.42e6)
    finally:
        plain.close()
    recorded = float(np.sum(g['losses']))
    assert abs(total - recorded) <= 3e-3 * recorded, (total, recorded)


def test_gradient_step_reproduces_the_recorded_second_iteration():
    """The tutorial's whole first FWI iteration through the product: the 15 shots' gradient (the
    plan's adjoint and imaging condition, undersampling 5 as the reference selects it for the
    processed wavelet), its processing on the inner grid (apply_prec, mask, smooth, norm), the
    slowness step of size 10 and the clip; then the recorded losses of the 15 shots of the second
    iteration at the updated model, each within 0.5 % (the oracle's chain: within 0.22 %).

    The recorded run injected the adjoint source as the reference's non-fw3d branch does,
    rec.inject(p_a, -rec[t-1] dt^2 vp^2) before the stencil (iso_acoustic/devito.py:750-751,
    793-794); this checkout forces the fw3d branch (:725), whose injection is the plan's. The older
    reading is the current one on the adjoint source delayed by two samples (it differs only by the
    first level's single injection; on this case the gradients agree to 7e-6)."""
    import torch
    from stride_gb300 import _lib
    from stride_gb300.pipelines import (Clip, FilterTraces, GradientDescent, MaskField, MuteTraces, NormField,
                                        NormPerShot, SmoothField, apply_prec)
    from oracle import numpy_oracle as npo

    g = T.load()
    dev = torch.device('cuda', torch.cuda.current_device())
    h, dt, nt = float(g['spacing']), float(g['dt']), int(g['nt'])
    e = [int(x) for x in g['extra']]
    geo = T.geometry(g)
    n_loc, n_shots = len(geo), len(g['shot_ids'])
    vp_true = torch.as_tensor(np.pad(g['vp_true'], [(e[0], e[0]), (e[1], e[1])], mode='edge'), device=dev)
    shape = tuple(vp_true.shape)
    inner = tuple(slice(a, s - a) for a, s in zip(e, shape))
    f = npo.select_undersampling(T.process_wavelet(T.wavelet(g), T.PERIOD_RECORDED)[None], dt)
    assert f == 5
    plan = _lib.Plan(2, shape, (h, h), tuple(e), tuple(int(x) for x in g['absorbing']), dt, nt, kernel='OT2',
                     density=_lib.SA_DENSITY_NONE, attenuation=False, undersampling=f, max_shots=n_shots)
    win = torch.as_tensor(npo.tukey(nt).astype(np.float32), device=dev)
    wav = torch.as_tensor(np.tile(T.wavelet(g)[None].astype(np.float32), (n_shots, 1)), device=dev)
    filt, mute, norm = FilterTraces(f_max=0.42e6), MuteTraces(f_max=0.42e6), NormPerShot()  # 31-tap tables
    offsets = np.arange(n_shots + 1) * n_loc
    eps = 1e-3 * h

    def geometry(shots):
        plan.set_geometry(np.arange(n_shots + 1), (geo[shots] + eps).astype(np.float32), offsets,
                          (np.tile(geo, (n_shots, 1)) + eps).astype(np.float32))

    def forward(vp, w, save=False):
        plan.set_medium(vp)
        out = torch.zeros((plan.n_rec, nt), device=dev)
        plan.forward((w * win[None]).contiguous(), out, save=save)
        return out

    def residual(modelled, obs_p):
        m, _ = mute.forward(modelled, obs_p, dt)
        m = filt.forward(m, dt=dt)
        o = filt.forward(obs_p, dt=dt)
        return norm.forward(m, offsets=offsets) - norm.forward(o, offsets=offsets)

    try:
        wav_p = filt.forward(wav, dt=dt)
        geometry(g['shot_ids'])
        obs_p = filt.forward(forward(vp_true, wav), dt=dt)
        vp = torch.full(shape, 1500., device=dev)
        res = residual(forward(vp, wav_p, save=True), obs_p)
        adj = filt.adjoint(res, dt=dt) * win[None]
        adj_s = torch.zeros_like(adj)
        adj_s[:, 2:] = adj[:, :-2]
        grad, prec = torch.zeros_like(vp), torch.zeros_like(vp)
        plan.adjoint(adj_s.contiguous(), grad, prec)
        d, _ = apply_prec((grad / vp)[inner].contiguous(), (prec / (vp * vp))[inner].contiguous())
        d = MaskField().forward(d, (slice(None), slice(None)))
        d = SmoothField().forward(d)
        d = NormField().forward(d, variable=vp, transform=lambda x: 1 / x)
        v = vp[inner].contiguous()
        GradientDescent(step_size=float(g['step_size'])).step(v, d)
        vp[inner] = v
        vp = Clip(min=float(g['clip'][0]), max=float(g['clip'][1])).forward(vp)
        geometry(g['shot_ids2'])
        obs_p = filt.forward(forward(vp_true, wav), dt=dt)
        res = residual(forward(vp, wav_p), obs_p).double()
    finally:
        plan.close()
    for k, s in enumerate(g['shot_ids2'].tolist()):
        got = 0.5 * float((res[k * n_loc:(k + 1) * n_loc] ** 2).sum())
        assert abs(got - g['losses2'][k]) <= 5e-3 * g['losses2'][k], (s, got, g['losses2'][k])
