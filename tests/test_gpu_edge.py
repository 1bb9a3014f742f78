"""Edge cases of the 2D plan through the C ABI: empty source/receiver sets, the shortest time axis,
points at the grid edge, re-used plans with a new geometry, and layout independence."""

import numpy as np
import pytest

from stride_gb300 import _lib
from tests import _cases as C

pytestmark = pytest.mark.gpu


def _plan(c, so, sx, ro, rx, **kw):
    plan = _lib.Plan(2, c['vp'].shape, c['spacing'], c['extra'], c['absorbing'], c['dt'], c['nt'], kernel='OT4',
                     density=C.density_mode(c['rho']), attenuation=c['alpha'] is not None, undersampling=4,
                     max_shots=kw.pop('max_shots', len(so) - 1), **kw)
    plan.set_medium(c['vp'], c['rho'], c['alpha'])
    plan.set_geometry(np.asarray(so), np.asarray(sx, np.float32), np.asarray(ro), np.asarray(rx, np.float32))
    return plan


def _wav(c, n):
    return np.ascontiguousarray(np.tile((c['wav'] * C.window(c['nt']))[None].astype(np.float32), (n, 1)))


def test_empty_point_sets():
    c = C.small_case(kernel='OT4', density='variable', alpha=True, n_shots=1, nt=160)
    eps = 1e-3 * np.asarray(c['spacing'])
    src = (np.asarray(c['srcs'][0], np.float32) + eps).astype(np.float32)
    rec = (np.asarray(c['recs'][0], np.float32) + eps).astype(np.float32)
    # shot 0: one source, no receivers; shot 1: no source, all receivers; shot 2: both
    so, ro = [0, 1, 1, 2], [0, 0, len(rec), 2 * len(rec)]
    plan = _plan(c, so, np.concatenate([src, src]), ro, np.concatenate([rec, rec]))
    tr = np.zeros((plan.n_rec, c['nt']), np.float32)
    plan.forward(_wav(c, 2), tr, save=True)
    assert np.all(tr[:len(rec)] == 0)            # shot 1 has no source
    ref, _ = C.oracle_forward(c, 0)
    assert C.rel_l2(tr[len(rec):], ref) <= 1e-4  # shot 2 is the one-shot case
    g = np.zeros(c['vp'].shape, np.float32)
    p = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(tr, g, p)
    assert np.isfinite(g).all()


def test_shortest_time_axis_and_bounds():
    c = C.small_case(kernel='OT4', density='none', n_shots=1, nt=40)
    c['nt'] = 3  # the reference's loop then runs a single step (time_m = time_M = 1)
    c['wav'] = c['wav'][:3]
    plan = C.make_plan(c)
    got, _ = C.gpu_forward(c, plan=plan)
    ref, _ = C.oracle_forward(c, 0)
    assert np.array_equal(got[0][:, [0, 2]], np.zeros((len(c['recs'][0]), 2), np.float32))
    assert C.rel_l2(got[0], ref) <= 1e-4 or np.abs(ref).max() == 0
    # points whose interpolation support leaves the grid are rejected
    nx, ny = c['vp'].shape
    h = c['spacing'][0]
    origin = -c['extra'][0] * h
    edge_ok = np.array([[origin + (nx - 2) * h + 0.4 * h, origin + 5.2 * h]], np.float32)
    edge_bad = np.array([[origin + (nx - 1) * h + 0.4 * h, origin + 5.2 * h]], np.float32)
    plan.set_geometry([0, 1], edge_ok, [0, 1], edge_ok)
    with pytest.raises(_lib.StrideAccError):
        plan.set_geometry([0, 1], edge_bad, [0, 1], edge_ok)
    hicks = C.make_plan(c, interpolation='hicks')
    with pytest.raises(_lib.StrideAccError):
        hicks.set_geometry([0, 1], edge_ok, [0, 1], edge_ok)  # 3 cells of support below, 4 above
    sinc = C.make_plan(c, interpolation='sinc')  # 6 cells of support below, 7 above
    near = np.array([[origin + 20.3 * h, origin + 5.2 * h]], np.float32)
    inside = np.array([[origin + 20.3 * h, origin + 6.2 * h]], np.float32)
    sinc.set_geometry([0, 1], inside, [0, 1], inside)
    with pytest.raises(_lib.StrideAccError):
        sinc.set_geometry([0, 1], near, [0, 1], inside)
    with pytest.raises(_lib.StrideAccError):  # more shots than the plan holds
        plan.set_geometry([0, 1, 2], np.concatenate([edge_ok, edge_ok]), [0, 1, 2], np.concatenate([edge_ok, edge_ok]))


def test_new_geometry_and_layout_independence():
    c = C.small_case(kernel='OT4', density='variable', alpha=True, n_shots=3, uneven=True, nt=200)
    fresh, _ = C.gpu_forward(c, plan=C.make_plan(c))
    # a plan built for more shots, first used with one shot, then re-targeted at the three
    plan = C.make_plan(c, max_shots=5)
    eps = 1e-3 * np.asarray(c['spacing'])

    def xyz(points):  # as make_plan forms them: FP32 coordinates plus the FP64 shift, stored as FP32
        return np.concatenate([np.asarray(p, np.float32) + eps for p in points]).astype(np.float32)

    plan.set_geometry([0, 1], xyz(c['srcs'][:1]), [0, len(c['recs'][0])], xyz(c['recs'][:1]))
    tr = np.zeros((plan.n_rec, c['nt']), np.float32)
    plan.forward(_wav(c, 1), tr)
    so = np.cumsum([0] + [len(s) for s in c['srcs']])
    ro = np.cumsum([0] + [len(r) for r in c['recs']])
    plan.set_geometry(so, xyz(c['srcs']), ro, xyz(c['recs']))
    again, _ = C.gpu_forward(c, plan=plan)
    plan.autotune()
    tuned, _ = C.gpu_forward(c, plan=plan)
    for a, b, d in zip(fresh, again, tuned):
        assert np.array_equal(a, b)
        assert np.array_equal(a, d)  # every point's arithmetic is the same in any launch shape


def test_autotune_cache_and_time_blocking_choice():
    """A second plan of the same shape takes the first one's tuned layout from the process cache;
    a single-shot plan, whose batch is too small for the streaming passes, is tuned to the
    persistent launch (every step in one launch) and its traces are unchanged bitwise."""
    c = C.small_case(kernel='OT4', density='variable', alpha=True, n_shots=1, nt=200)
    plan = C.make_plan(c)
    plan.set_option(_lib.SA_OPT_PERSISTENT, -1)
    streaming, _ = C.gpu_forward(c, plan=plan)
    plan.set_option(_lib.SA_OPT_PERSISTENT, 0)
    plan.autotune()
    tuned, _ = C.gpu_forward(c, plan=plan)
    assert plan.launches <= 3  # the persistent launch won
    assert np.array_equal(tuned[0], streaming[0])
    twin = C.make_plan(c)
    C.gpu_forward(c, plan=twin)
    twin.autotune()
    assert twin.layout == plan.layout


def test_autotune_refuses_to_discard_a_saved_wavefield():
    """sa_autotune steps the plan's wavefield buffers: between a saving forward and its adjoint it
    returns SA_E_INVALID and the saved wavefield still gives the untuned gradient."""
    c = C.small_case(kernel='OT4', density='none', n_shots=2, nt=160)
    plan = C.make_plan(c)
    got, plan = C.gpu_forward(c, plan=plan, save=True)
    with pytest.raises(_lib.StrideAccError) as e:
        plan.autotune()
    assert e.value.code == _lib.SA_E_INVALID
    res = np.ascontiguousarray(np.concatenate(got) * np.float32(0.5))
    g1 = np.zeros(c['vp'].shape, np.float32)
    p1 = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(res, g1, p1)
    plan.autotune()  # the saved wavefield has been used: allowed again
    C.gpu_forward(c, plan=plan, save=True)
    g2 = np.zeros(c['vp'].shape, np.float32)
    p2 = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(res, g2, p2)
    assert np.array_equal(g1, g2) and np.array_equal(p1, p2)
