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
