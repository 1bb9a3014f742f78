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
