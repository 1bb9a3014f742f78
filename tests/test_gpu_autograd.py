"""torch.autograd around the CUDA forward map (stride_gb300.autograd.WaveOperator): the backward
is the exact discrete adjoint, checked against the FP64 oracle, against central finite
differences of the misfit and across interleaved forwards (checkpoints rebuilt on demand)."""

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import numpy_oracle as npo  # noqa: E402
from tests import _cases as C  # noqa: E402

pytestmark = pytest.mark.gpu


def _operator(c, **kw):
    from stride_gb300.autograd import WaveOperator
    eps = 1e-3 * np.asarray(c['spacing'])
    so = np.cumsum([0] + [len(s) for s in c['srcs']])
    ro = np.cumsum([0] + [len(r) for r in c['recs']])
    sx = np.concatenate([np.asarray(s, np.float32) + eps for s in c['srcs']]).astype(np.float32)
    rx = np.concatenate([np.asarray(r, np.float32) + eps for r in c['recs']]).astype(np.float32)
    wav = np.concatenate([np.tile(c['wav'][None], (len(s), 1)) for s in c['srcs']]).astype(np.float64)
    wav = (wav * C.window(c['nt'])[None, :]).astype(np.float32)
    return WaveOperator(c['vp'].shape, c['spacing'], c['extra'], c['absorbing'], c['dt'], c['nt'], so, sx, ro, rx, wav,
                        rho=c['rho'], alpha=c['alpha'], kernel=c['kernel'], **kw)


def test_autograd_gradient_oracle_and_finite_differences():
    ndimage = pytest.importorskip('scipy.ndimage')
    c = C.small_case(kernel='OT4', density='variable', alpha=True, inner=40, nt=200, n_shots=2, uneven=True)
    op = _operator(c, checkpoint_interval=25)
    dev = op.device
    obs = op(torch.as_tensor(c['vp'], device=dev)).detach()
    vp0 = torch.full(c['vp'].shape, 1500., device=dev, requires_grad=True)
    misfit = 0.5 * ((op(vp0) - obs) ** 2).sum()
    misfit.backward()
    g = vp0.grad.cpu().numpy()
    # oracle: exact adjoint of each shot with its residual
    res = (op(vp0.detach()) - obs).cpu().numpy().astype(np.float64)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    ref = np.zeros(c['vp'].shape)
    k = 0
    for s in range(2):
        nr = len(c['recs'][s])
        gs, _ = npo.adjoint_exact(np.full(c['vp'].shape, 1500.), c['spacing'], c['dt'], c['nt'], c['absorbing'],
                                  c['srcs'][s], c['recs'][s], np.tile(c['wav'][None], (len(c['srcs'][s]), 1)),
                                  res[k:k + nr], origin, rho=c['rho'], alpha=c['alpha'], kernel='OT4')
        ref += gs
        k += nr
    assert C.cosine(g, ref) >= 0.99999
    assert C.rel_l2(g, ref) <= 2e-3
    rng = np.random.default_rng(4)
    with torch.no_grad():
        J = lambda v: 0.5 * float(((op(v) - obs).double() ** 2).sum())
        fds, ans = [], []
        for _ in range(8):
            d = ndimage.gaussian_filter(rng.standard_normal(c['vp'].shape), 3)
            d = torch.as_tensor(d / np.abs(d).max(), dtype=torch.float32, device=dev)
            fds.append((J(vp0 + d) - J(vp0 - d)) / 2)
            ans.append(float((vp0.grad.double() * d.double()).sum()))
    fds, ans = np.array(fds), np.array(ans)
    assert np.linalg.norm(fds - ans) <= 1e-2 * np.linalg.norm(fds), (fds, ans)


def test_backward_after_another_forward():
    c = C.small_case(kernel='OT4', density='none', inner=40, nt=160, n_shots=1)
    op = _operator(c, checkpoint_interval=16)
    dev = op.device
    w = torch.as_tensor(np.random.default_rng(2).standard_normal((op.n_rec, c['nt'])), dtype=torch.float32,
                        device=dev)
    v1 = torch.as_tensor(c['vp'], device=dev).requires_grad_(True)
    (op(v1) * w).sum().backward()
    g_alone = v1.grad.clone()
    v1.grad = None
    t1 = op(v1)
    op(torch.full_like(v1, 1500.))  # replaces the plan's checkpoints
    (t1 * w).sum().backward()
    assert torch.equal(v1.grad, g_alone)
