"""GPU trace and field processing (stride_gb300.pipelines over csrc/pipelines.cu) against the
NumPy/SciPy restatement of the reference's pipeline steps on identical seeded inputs."""

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import pipelines_oracle as PO  # noqa: E402
from tests import _cases as C  # noqa: E402

pytestmark = pytest.mark.gpu

DT = 9.09e-8


def _traces(n=37, nt=900, seed=0):
    rng = np.random.default_rng(seed)
    t = np.arange(nt) * DT
    x = np.zeros((n, nt), np.float32)
    for i in range(n):
        f = rng.uniform(0.3e6, 2.5e6)
        x[i] = (np.sin(2 * np.pi * f * t + rng.uniform(0, 6)) * np.exp(-((t - rng.uniform(0.2, 0.6) * t[-1]) / 8e-6) ** 2)
                + 0.1 * rng.standard_normal(nt)).astype(np.float32)
    return x


def _dev(x):
    return torch.as_tensor(np.ascontiguousarray(x), device='cuda')


@pytest.mark.parametrize('f_min,f_max,ftype', [(None, 1.5e6, None), (0.3e6, 1.5e6, None), (0.4e6, None, None),
                                               (None, 1.5e6, 'butterworth'), (None, 1.2e6, 'fir'),
                                               (0.3e6, 1.8e6, 'fir')])
def test_filter_traces(f_min, f_max, ftype):
    from stride_gb300.pipelines import FilterTraces
    x = _traces()
    op = FilterTraces(f_min=f_min, f_max=f_max, filter_type=ftype)
    got = op.forward(_dev(x), dt=DT).cpu().numpy()
    if ftype == 'fir':  # the oracle restates the causal FIR filters with lfilter
        lo = f_min * DT if f_min is not None else 0
        hi = f_max * DT
        order, beta = PO.scipy.signal.kaiserord(30, 0.050)
        order = order // 2 * 2 + 1
        cutoff = hi / 0.5 if f_min is None else [lo / 0.5, hi / 0.5]
        b = PO.scipy.signal.firwin(order, cutoff, pass_zero='lowpass' if f_min is None else 'bandpass',
                                   window=('kaiser', beta), scale=True)
        ref = PO.scipy.signal.lfilter(b, 1., x, axis=-1).astype(np.float32)
    else:
        ref = PO.filter_traces(x, DT, f_min=f_min, f_max=f_max, filter_type=ftype)
    assert C.rel_l2(got, ref) <= 1e-6
    # adjoint: <F x, y> = <x, F^T y>
    y = _traces(seed=1)
    fx = op.forward(_dev(x), dt=DT).double()
    op.forward(_dev(x), dt=DT)
    fty = op.adjoint(_dev(y), dt=DT).double()
    lhs = float((fx * _dev(y).double()).sum())
    rhs = float((_dev(x).double() * fty).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_norm_mute_check():
    from stride_gb300.pipelines import CheckTraces, MuteTraces, NormPerShot
    x = _traces(n=50)
    offsets = [0, 20, 20, 50]  # uneven, with an empty shot
    got = NormPerShot().forward(_dev(x), offsets=offsets).cpu().numpy()
    ref = np.concatenate([PO.norm_per_shot(x[a:b]) for a, b in zip(offsets[:-1], offsets[1:]) if b > a])
    assert C.rel_l2(got, ref) <= 1e-6
    obs = _traces(n=50, seed=3)
    obs[:, :100] = 0
    obs[7, 400:460] = 0
    mod = _traces(n=50, seed=4)
    m_got, _ = MuteTraces(f_max=1.5e6).forward(_dev(mod), _dev(obs), DT)
    m_ref = PO.mute_traces(mod, obs, DT, f_max=1.5e6)
    assert C.rel_l2(m_got.cpu().numpy(), m_ref) <= 1e-6
    bad = x.copy()
    bad[3, 10] = np.nan
    bad[9, 0] = np.inf
    with pytest.raises(RuntimeError):
        CheckTraces().forward(_dev(bad))
    cleaned = CheckTraces(raise_incorrect=False, filter_incorrect=True).forward(_dev(bad)).cpu().numpy()
    assert np.all(cleaned[3] == 0) and np.all(cleaned[9] == 0) and np.array_equal(cleaned[4], x[4])


def test_field_steps():
    from stride_gb300.pipelines import Clip, GradientDescent, MaskField, NormField, SmoothField, apply_prec
    rng = np.random.default_rng(5)
    shape = (96, 83)
    inner = (slice(20, 76), slice(20, 63))
    g = rng.standard_normal(shape).astype(np.float32)
    got = MaskField(mask_rampoff=10).forward(_dev(g), inner).cpu().numpy()
    assert np.array_equal(got, g * PO.field_mask(shape, inner, 10))
    for sigma in (0.25, 1.7, (0.5, 2.0)):
        got = SmoothField(smooth_sigma=sigma).forward(_dev(g)).cpu().numpy()
        assert C.rel_l2(got, PO.smooth_field(g, sigma)) <= 1e-6
    vp = (1500 + 100 * rng.random(shape)).astype(np.float32)
    got = NormField().forward(_dev(g), variable=_dev(vp)).cpu().numpy()
    assert C.rel_l2(got, PO.norm_field(g, vp)) <= 1e-6
    got = Clip(min=-0.5, max=0.7).forward(_dev(g)).cpu().numpy()
    assert np.array_equal(got, np.clip(g, -0.5, 0.7))
    prec = np.abs(rng.standard_normal(shape)).astype(np.float32) * 1e3
    gg, pp = apply_prec(_dev(g), _dev(prec))
    g_ref, p_ref = PO.apply_prec(g, prec)
    assert C.rel_l2(pp.cpu().numpy(), p_ref) <= 1e-5
    assert C.rel_l2(gg.cpu().numpy(), g_ref) <= 1e-5
    d = rng.standard_normal(shape).astype(np.float32) * 1e-6
    v = _dev(vp)
    GradientDescent(step_size=0.3).step(v, _dev(d))
    ref = 1 / (1 / vp - np.float32(0.3) * d)
    assert C.rel_l2(v.cpu().numpy(), ref) <= 1e-6
