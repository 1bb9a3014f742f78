"""Plain FWI on the GPU (stride_gb300.fwi.PlainFWI): the reference's inversion loop with batched
shots and GPU pipelines reduces the vp error of a seeded phantom."""

import numpy as np
import pytest

torch = pytest.importorskip('torch')

pytestmark = pytest.mark.gpu


def test_plain_fwi_reduces_error():
    from stride_gb300 import phantoms
    from stride_gb300.fwi import PlainFWI
    w = phantoms.workload('single', seed=1, nt=700, inner=96)
    shots = list(range(0, 128, 8))
    w['shots'] = shots
    w['src'] = [w['geometry'][[s]] for s in shots]
    w['rec'] = [w['geometry'] for _ in shots]
    fwi = PlainFWI(w, step_size=2.)
    e0 = fwi.error()
    errs = [fwi.iterate(f_max=0.4e6)['error'] for _ in range(6)]
    fwi.close()
    assert np.all(np.isfinite(errs))
    assert np.all(np.diff([e0] + errs) < 0), (e0, errs)  # every iteration moves towards the true model
    assert errs[-1] < 0.9 * e0, (e0, errs)


def test_learned_fwi_runs_and_falls_back():
    """Pairs from plain-FWI paths, a few U-Net epochs, then learned iterations: every step either
    lowers the misfit with the network's update or is the plain step."""
    from stride_gb300 import phantoms
    from stride_gb300.fwi import LearnedFWI, PlainFWI, generate_pairs, train_unet
    from stride_gb300.unet import UNet

    def wl(seed):
        w = phantoms.workload('single', seed=seed, nt=600, inner=128)
        shots = list(range(0, 128, 16))
        w['shots'] = shots
        w['src'] = [w['geometry'][[s]] for s in shots]
        w['rec'] = [w['geometry'] for _ in shots]
        return w

    plain = PlainFWI(wl(10), step_size=2.)
    X, T = generate_pairs(plain, [wl(10 + i)['vp'] for i in range(2)], iterations=2, f_max=0.4e6)
    assert tuple(X.shape) == (4, 128, 128, 2) and tuple(T.shape) == (4, 128, 128)
    net = UNet(seed=0)
    losses = train_unet(net, X, T, epochs=3, batch=2)
    assert np.all(np.isfinite(losses)) and net.errors() == 0
    learned = LearnedFWI(wl(0), net, step_size=2.)
    for _ in range(3):
        m0 = learned.misfit(learned.vp, 0.4e6)
        rec = learned.iterate(0.4e6)
        assert np.isfinite(rec['error'])
        if rec['learned']:
            assert learned.misfit(learned.vp, 0.4e6) < m0
    plain.close()
    learned.close()
