"""The persistent forward of small batches (one cooperative launch runs every step,
stride_gb300/csrc/persist2d.cu): its traces equal the streaming step passes' bit for bit for every
operator variant and for uneven batches; the single-shot workload matches the oracle; and halo
waits that cannot complete (the tests' option makes each wait ask for a level one beyond what any
tile publishes) give up within their bound: sa_forward returns SA_E_TIMEOUT and the plan keeps
working."""

import numpy as np
import pytest

from stride_gb300 import _lib
from tests import _cases as C

pytestmark = pytest.mark.gpu


def _forward(c, plan, mode):
    plan.set_option(_lib.SA_OPT_PERSISTENT, mode)
    got, _ = C.gpu_forward(c, plan=plan)
    return np.concatenate(got)


@pytest.mark.parametrize('kernel', ['OT2', 'OT4'])
@pytest.mark.parametrize('density,alpha', [('none', False), ('variable', True), ('constant', False)])
def test_persistent_equals_streaming(kernel, density, alpha):
    c = C.small_case(kernel=kernel, density=density, alpha=alpha, n_shots=3, uneven=True, nt=220)
    plan = C.make_plan(c)
    streaming = _forward(c, plan, -1)
    persistent = _forward(c, plan, 1)
    assert plan.launches <= 3  # wavelet transpose, the persistent launch, trace transpose
    assert np.abs(streaming).max() > 0
    assert np.array_equal(persistent, streaming)


@pytest.mark.parametrize('kernel', ['OT2', 'OT4'])
def test_persistent_crowded_tiles_equal_streaming(kernel):
    """Sources and receivers crowded into a few tiles: a CTA with more source targets than its
    shared-memory slots adds them in a pass of its own, and one with more receivers than threads
    gathers the rest from global memory."""
    c = C.small_case(kernel=kernel, density='variable', alpha=True, n_shots=2, nt=160)
    rng = np.random.default_rng(5)
    h = c['spacing'][0]
    centre = np.array([20 * h, 24 * h])
    c['srcs'] = [centre + rng.uniform(0, 6 * h, (48, 2)) for _ in range(2)]  # 4 targets each, ~190 per pair
    c['recs'] = [centre + rng.uniform(0, 10 * h, (600, 2)) for _ in range(2)]
    plan = C.make_plan(c)
    streaming = _forward(c, plan, -1)
    persistent = _forward(c, plan, 1)
    assert np.abs(streaming).max() > 0
    assert np.array_equal(persistent, streaming)


def test_persistent_single_shot_workload_matches_oracle():
    """The single-shot workload (256^2 inner at 0.5 mm, 2000 steps, 128 receivers) runs the
    persistent forward by default."""
    from stride_gb300 import phantoms
    w = phantoms.workload('single')
    c = dict(vp=w['vp'], rho=None, alpha=None, spacing=w['spacing'], dt=w['dt'], nt=w['nt'], extra=w['extra'],
             absorbing=w['absorbing'], kernel='OT4', srcs=w['src'], recs=w['rec'], wav=w['wavelet'])
    plan = C.make_plan(c)
    got, _ = C.gpu_forward(c, plan=plan)
    assert plan.launches <= 3
    ref, _ = C.oracle_forward(c, 0)
    assert C.rel_l2(got[0], ref) <= 1e-4


def test_wait_timeout_is_reported_and_the_plan_recovers():
    c = C.small_case(kernel='OT4', density='variable', alpha=True, n_shots=2, nt=120)
    plan = C.make_plan(c)
    good = _forward(c, plan, 1)
    plan.set_option(_lib.SA_OPT_BARRIER_SPIN, 20000)  # milliseconds per wait
    plan.set_option(_lib.SA_OPT_BARRIER_EXTRA, 1)     # a level beyond every tile's: no wait can complete
    with pytest.raises(_lib.StrideAccError) as e:
        _forward(c, plan, 1)
    assert e.value.code == _lib.SA_E_TIMEOUT
    plan.set_option(_lib.SA_OPT_BARRIER_EXTRA, 0)
    plan.set_option(_lib.SA_OPT_BARRIER_SPIN, 10_000_000)
    assert np.array_equal(_forward(c, plan, 1), good)


def test_option_values_are_checked():
    c = C.small_case(kernel='OT4', density='none', n_shots=1, nt=60)
    plan = C.make_plan(c)
    for option, value in ((_lib.SA_OPT_PERSISTENT, 2), (_lib.SA_OPT_BARRIER_EXTRA, -1), (_lib.SA_OPT_BARRIER_SPIN, 0),
                          (99, 0)):
        with pytest.raises(_lib.StrideAccError) as e:
            plan.set_option(option, value)
        assert e.value.code == _lib.SA_E_INVALID
