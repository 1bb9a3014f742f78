"""Parity at the benchmarked sizes: the CUDA path (through the C ABI) against the C oracle on the
bench's own workloads, not on reduced cases.

* The fwd+adj vp-gradient workload (552^2 extended, vp/rho/alpha phantom, jittered transducers,
  4000 steps, OT4, f = 4) for 2 of its shots: observed traces on the true phantom, traces on the
  1500 m/s starting model, then the reference imaging-condition gradient and preconditioner of
  the L2 residual. Traces relative L2 <= 1e-4, gradient cosine >= 0.999 and relative L2 <= 1e-3,
  preconditioner relative L2 <= 1e-4 (FP32 throughout).
* The batched forward workload (same grid and phantom) run as a 16-shot batch, the first and last
  shots compared with the oracle (traces relative L2 <= 1e-4).
* The same 2-shot gradient with the forward wavefield checkpointed every 50 steps and recomputed:
  bitwise equal to the gradient from the full undersampled wavefield.
* The exact gradient of the misfit at full size against central finite differences of the CUDA
  forward on 32 smooth random vp directions (relative error <= 1e-2).
"""

import numpy as np
import pytest

from tests import _cases as C

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-4


def _case(workload, n_shots, vp=None):
    import bench
    w = bench.workload_config(workload, n_shots=n_shots)
    return dict(vp=w['vp'] if vp is None else vp, rho=w['rho'], alpha=w['alpha'], spacing=w['spacing'], dt=w['dt'],
                nt=w['nt'], extra=w['extra'], absorbing=w['absorbing'], kernel='OT4', srcs=w['src'], recs=w['rec'],
                wav=w['wavelet'])


def _wavelets(c):
    wav = np.concatenate([np.tile(c['wav'][None], (len(s), 1)) for s in c['srcs']]).astype(np.float64)
    return np.ascontiguousarray((wav * C.window(c['nt'])[None, :]).astype(np.float32))


def _start(c):
    """The workload's starting model: 1500 m/s everywhere, the true rho and alpha."""
    return dict(c, vp=np.full(c['vp'].shape, 1500., np.float32))


def _residual_gradient(plan, c0, obs, save=True):
    """GPU traces at c0, the residual against obs, and its parity gradient (C ABI, host buffers)."""
    tr = np.zeros_like(obs)
    plan.forward(_wavelets(c0), tr, save=save)
    res = (tr - obs).astype(np.float32)
    resw = np.ascontiguousarray((res.astype(np.float64) * C.window(c0['nt'])[None, :]).astype(np.float32))
    grad = np.zeros(c0['vp'].shape, np.float32)
    prec = np.zeros(c0['vp'].shape, np.float32)
    plan.adjoint(resw, grad, prec)
    return tr, res, grad, prec


def test_gradient_workload_two_shots_full_size():
    c = _case('fwdadj64', 2)
    assert c['vp'].shape == (552, 552) and c['nt'] == 4000 and len(c['srcs']) == 2
    plan = C.make_plan(c)
    obs, _ = C.gpu_forward(c, plan=plan)
    for s in range(2):
        ref, _ = C.oracle_forward(c, s)
        assert np.abs(ref).max() > 0
        assert C.rel_l2(obs[s], ref) <= TRACE_TOL, s
    obs = np.ascontiguousarray(np.concatenate(obs))
    c0 = _start(c)
    plan.set_medium(c0['vp'], c0['rho'], c0['alpha'])
    tr, res, grad, prec = _residual_gradient(plan, c0, obs)
    g_ref = np.zeros(c['vp'].shape, np.float64)
    p_ref = np.zeros(c['vp'].shape, np.float64)
    k = 0
    for s in range(2):
        nr = len(c0['recs'][s])
        ref, snaps = C.oracle_forward(c0, s, save=True)
        assert C.rel_l2(tr[k:k + nr], ref) <= TRACE_TOL, s
        g, p = C.oracle_adjoint(c0, s, res[k:k + nr], snaps)
        del snaps
        g_ref += g
        p_ref += p
        k += nr
    assert np.isfinite(grad).all() and np.abs(g_ref).max() > 0
    assert C.cosine(grad, g_ref) >= 0.999
    assert C.rel_l2(grad, g_ref) <= 1e-3
    assert C.rel_l2(prec, p_ref) <= 1e-4


def test_batched_forward_workload_full_size():
    c = _case('fwd256', 16)
    assert c['vp'].shape == (552, 552) and c['nt'] == 4000 and len(c['srcs']) == 16
    got, _ = C.gpu_forward(c)
    for s in (0, 15):
        ref, _ = C.oracle_forward(c, s)
        assert C.rel_l2(got[s], ref) <= TRACE_TOL, s


def test_checkpointed_gradient_full_size_bitwise():
    """The gradient workload's wavefield checkpointed every 50 steps with recompute gives the
    snapshot path's gradient and preconditioner bit for bit."""
    c = _case('fwdadj64', 2)
    plan = C.make_plan(c)
    obs = np.zeros((plan.n_rec, c['nt']), np.float32)
    plan.forward(_wavelets(c), obs)
    c0 = _start(c)
    plan.set_medium(c0['vp'], c0['rho'], c0['alpha'])
    tr0, _, g0, p0 = _residual_gradient(plan, c0, obs)
    assert np.abs(g0).max() > 0
    plan_ck = C.make_plan(c0, checkpoint_interval=50)
    tr1, _, g1, p1 = _residual_gradient(plan_ck, c0, obs, save='checkpoints')
    assert np.array_equal(tr0, tr1)
    assert np.array_equal(g0, g1)
    assert np.array_equal(p0, p1)


def test_exact_gradient_central_differences_full_size():
    """Misfit J = 1/2 ||traces(vp) - observed||^2 of 4 shots of the gradient workload through the
    CUDA forward; its exact gradient (checkpoints every 50 steps) against central differences on
    32 smooth random directions (white noise smoothed over 3 cells, peak 1 m/s per unit step)."""
    ndimage = pytest.importorskip('scipy.ndimage')
    c = _case('fwdadj64', 4)
    plan = C.make_plan(c, checkpoint_interval=50)
    obs = np.zeros((plan.n_rec, c['nt']), np.float32)
    plan.forward(_wavelets(c), obs)
    vp0 = np.full(c['vp'].shape, 1500., np.float32)

    def misfit(vp):
        plan.set_medium(np.ascontiguousarray(vp.astype(np.float32)), c['rho'], c['alpha'])
        tr = np.zeros_like(obs)
        plan.forward(_wavelets(c), tr)
        return 0.5 * float(np.sum((tr.astype(np.float64) - obs) ** 2))

    plan.set_medium(vp0, c['rho'], c['alpha'])
    tr = np.zeros_like(obs)
    plan.forward(_wavelets(c), tr, save='checkpoints')
    g = np.zeros(vp0.shape, np.float32)
    p = np.zeros(vp0.shape, np.float32)
    plan.adjoint(np.ascontiguousarray((tr.astype(np.float64) - obs).astype(np.float32)), g, p, exact=True)
    assert np.isfinite(g).all() and np.abs(g).max() > 0
    rng = np.random.default_rng(12)
    fds, ans = [], []
    for _ in range(32):
        d = ndimage.gaussian_filter(rng.standard_normal(vp0.shape), 3)
        d /= np.abs(d).max()
        eps = 1.0
        fds.append((misfit(vp0 + eps * d) - misfit(vp0 - eps * d)) / (2 * eps))
        ans.append(float(np.sum(g.astype(np.float64) * d)))
    fds, ans = np.array(fds), np.array(ans)
    assert np.linalg.norm(fds - ans) <= 1e-2 * np.linalg.norm(fds), (fds, ans)
    assert np.all(np.abs(fds - ans) <= 1e-2 * np.sqrt(np.mean(fds ** 2))), (fds, ans)
