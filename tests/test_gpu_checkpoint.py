"""Wavefield checkpointing (SA_SAVE_CHECKPOINTS): the adjoint that recomputes each segment's
snapshots from stored checkpoints returns the same gradient and preconditioner, bit for bit,
as the adjoint from the full undersampled wavefield, in 2D and 3D, for intervals that divide
the adjoint's time range, that do not, that cover it in one segment, for an interval chosen
from a byte budget, with the CFS-PML (its auxiliary fields checkpointed with the levels), and
with the two-level schedule a budget below every one-level schedule selects (fine checkpoints
placed by a recompute of each coarse segment)."""

import numpy as np
import pytest

from stride_gb300 import _lib
from tests import _cases as C
from tests.test_gpu_3d import case3d, make_plan3

pytestmark = pytest.mark.gpu


def _residuals(c, got):
    rng = np.random.default_rng(5)
    res = [rng.standard_normal(g.shape).astype(np.float32) * np.abs(g).max() for g in got]
    return np.ascontiguousarray((np.concatenate(res).astype(np.float64) * C.window(c['nt'])[None, :])
                                .astype(np.float32))


def _gradient(c, plan, save, resw=None):
    got, plan = C.gpu_forward(c, plan=plan, save=save)
    if resw is None:
        resw = _residuals(c, got)
    grad = np.zeros(c['vp'].shape, np.float32)
    prec = np.zeros(c['vp'].shape, np.float32)
    plan.adjoint(resw, grad, prec)
    return np.concatenate(got), grad, prec, resw


@pytest.mark.parametrize('interval', [4, 20, 36, 1000])
def test_checkpointed_gradient_2d_bitwise(interval):
    c = C.small_case(kernel='OT4', density='variable', alpha=True, n_shots=3, uneven=True, nt=250)
    tr0, g0, p0, resw = _gradient(c, C.make_plan(c), True)
    assert np.abs(g0).max() > 0
    plan = C.make_plan(c, checkpoint_interval=interval)
    tr1, g1, p1, _ = _gradient(c, plan, 'checkpoints', resw)
    assert np.array_equal(tr0, tr1)
    assert np.array_equal(g0, g1)
    assert np.array_equal(p0, p1)
    # replayed graphs give the same result again
    _, g2, _, _ = _gradient(c, plan, 'checkpoints', resw)
    assert np.array_equal(g0, g2)


def test_checkpoint_budget_2d():
    c = C.small_case(kernel='OT4', density='none', n_shots=2, nt=300)
    _, g0, _, resw = _gradient(c, C.make_plan(c), True)
    level = 2 * c['vp'].shape[0] * ((c['vp'].shape[1] + 2 + 31) // 32 * 32) * 4  # one level of a shot pair
    plan = C.make_plan(c, checkpoint_interval=8, checkpoint_budget=30 * level)
    _, g1, _, _ = _gradient(c, plan, 'checkpoints', resw)
    assert np.array_equal(g0, g1)
    bad = C.make_plan(c, checkpoint_interval=8, checkpoint_budget=2 * level)
    with pytest.raises(_lib.StrideAccError) as e:
        _gradient(c, bad, 'checkpoints', resw)
    assert e.value.code == _lib.SA_E_NOMEM


def test_adjoint_follows_latest_saving_forward():
    c = C.small_case(kernel='OT4', density='none', n_shots=1, nt=200)
    plan = C.make_plan(c, checkpoint_interval=12)
    _, g_ck, _, resw = _gradient(c, plan, 'checkpoints')
    _, g_sn, _, _ = _gradient(c, plan, True, resw)
    assert np.array_equal(g_ck, g_sn)
    # a forward without saving leaves nothing to recompute from
    plan2 = C.make_plan(c, checkpoint_interval=12)
    C.gpu_forward(c, plan=plan2, save='checkpoints')
    C.gpu_forward(c, plan=plan2, save=False)
    with pytest.raises(_lib.StrideAccError):
        plan2.adjoint(resw, np.zeros(c['vp'].shape, np.float32), np.zeros(c['vp'].shape, np.float32))


@pytest.mark.parametrize('interval', [8, 44])
def test_checkpointed_gradient_3d_bitwise(interval):
    c = case3d(kernel='OT4', density='variable', alpha=True, n_shots=2, nt=150)
    tr0, g0, p0, resw = _gradient(c, make_plan3(c), True)
    assert np.abs(g0).max() > 0
    tr1, g1, p1, _ = _gradient(c, make_plan3(c, checkpoint_interval=interval), 'checkpoints', resw)
    assert np.array_equal(tr0, tr1)
    assert np.array_equal(g0, g1)
    assert np.array_equal(p0, p1)


@pytest.mark.parametrize('interval', [12, 40])
def test_checkpointed_gradient_pml_2d_bitwise(interval):
    c = C.small_case(kernel='OT2', density='variable', alpha=True, n_shots=3, uneven=True, nt=220, inner=40)
    kw = dict(boundary='pml', f_centre=1.0e6)
    tr0, g0, p0, resw = _gradient(c, C.make_plan(c, **kw), True)
    assert np.abs(g0).max() > 0
    plan = C.make_plan(c, checkpoint_interval=interval, **kw)
    tr1, g1, p1, _ = _gradient(c, plan, 'checkpoints', resw)
    assert np.array_equal(tr0, tr1)
    assert np.array_equal(g0, g1)
    assert np.array_equal(p0, p1)
    _, g2, _, _ = _gradient(c, plan, 'checkpoints', resw)
    assert np.array_equal(g0, g2)


def test_checkpointed_gradient_pml_3d_bitwise():
    c = case3d(kernel='OT2', density='variable', alpha=True, n_shots=2, nt=120)
    kw = dict(boundary='pml', f_centre=1.0e6)
    tr0, g0, p0, resw = _gradient(c, make_plan3(c, **kw), True)
    assert np.abs(g0).max() > 0
    tr1, g1, p1, _ = _gradient(c, make_plan3(c, checkpoint_interval=16, **kw), 'checkpoints', resw)
    assert np.array_equal(tr0, tr1)
    assert np.array_equal(g0, g1)
    assert np.array_equal(p0, p1)


def _least_one_level(nt, level, ck_levels=2, f=4):
    """Least bytes of a one-level schedule: (nt-2)/K checkpoints of ck_levels levels and one
    segment of K/f snapshot levels, K a multiple of f up to nt-1-f."""
    return min(((nt - 2) // k) * ck_levels * level + (k // f) * level for k in range(f, nt - f, f))


def _two_level(c, make, level, ck_levels=2, **kw):
    """Gradients of the snapshot path, a one-level schedule and a budget that forces two levels."""
    tr0, g0, p0, resw = _gradient(c, make(c, **kw), True)
    assert np.abs(g0).max() > 0
    one = make(c, checkpoint_interval=40, **kw)
    _gradient(c, one, 'checkpoints', resw)
    budget = 0.9 * _least_one_level(c['nt'], level, ck_levels)
    two = make(c, checkpoint_interval=40, checkpoint_budget=budget, **kw)
    tr1, g1, p1, _ = _gradient(c, two, 'checkpoints', resw)
    return (tr0, g0, p0), (tr1, g1, p1), one, two, resw


def test_two_level_checkpoints_2d_bitwise():
    c = C.small_case(kernel='OT4', density='variable', alpha=True, n_shots=3, uneven=True, nt=250)
    nx, ny = c['vp'].shape
    level = 2 * nx * ((ny + 2 + 31) // 32 * 32) * 8  # one level of both shot pairs (float2)
    ref, got, one, two, resw = _two_level(c, C.make_plan, level)
    assert two.launches > one.launches  # the recompute that places the fine checkpoints
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
    shape = c['vp'].shape
    with pytest.raises(_lib.StrideAccError) as e:  # the exact gradient's schedule has one level
        two.adjoint(resw, np.zeros(shape, np.float32), np.zeros(shape, np.float32), exact=True)
    assert e.value.code == _lib.SA_E_NOMEM
    bad = C.make_plan(c, checkpoint_interval=40, checkpoint_budget=4 * level)
    with pytest.raises(_lib.StrideAccError) as e:
        _gradient(c, bad, 'checkpoints', resw)
    assert e.value.code == _lib.SA_E_NOMEM


def test_two_level_checkpoints_pml_2d_bitwise():
    c = C.small_case(kernel='OT2', density='variable', alpha=True, n_shots=2, nt=220, inner=40)
    nx, ny = c['vp'].shape
    level = nx * ((ny + 2 + 31) // 32 * 32) * 8
    ref, got, one, two, _ = _two_level(c, C.make_plan, level, ck_levels=8, boundary='pml', f_centre=1.0e6)
    assert two.launches > one.launches
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)


def test_two_level_checkpoints_3d_bitwise():
    c = case3d(kernel='OT4', density='variable', alpha=True, n_shots=2, nt=130)
    nx, ny, nz = c['vp'].shape
    level = 2 * nx * ny * ((nz + 2 + 31) // 32 * 32) * 4  # one level of both shots
    ref, got, one, two, _ = _two_level(c, make_plan3, level)
    assert two.launches > one.launches
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)
