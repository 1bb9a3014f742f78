"""The oracle's chain through both recorded iterations of the reference's imaging tutorial
(run: python tests/golden/check_tutorial_oracle.py; about 5 minutes on 8 cores, which is why it is
not part of the CPU test suite; tests/test_pin_tutorial.py runs the first iteration on 3 shots and
tests/test_gpu_tutorial.py the product's chain through both).

Iteration 1: the 15 recorded shots at vp = 1500 m/s; each shot's loss, its adjoint source (the
filter's adjoint; norm and mute pass through, as in the reference) and its gradient, the older
adjoint injection reading as the current one on the source delayed by two samples. The summed
gradient's processing on the inner grid (get_grad_vp's slowness chain rule, Data.apply_prec,
MaskField, SmoothField, NormField), the slowness step and the clip give the model of iteration 2,
whose 15 recorded losses are then compared. Exits 1 if a loss differs by more than 0.3 %.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import c_oracle  # noqa: E402
from oracle import numpy_oracle as npo  # noqa: E402
from oracle import pipelines_oracle as pipes  # noqa: E402
from tests import _tutorial as T  # noqa: E402

TOL = 3e-3


def main():
    g = T.load()
    per = T.PERIOD_RECORDED
    w = T.wavelet(g)
    wp = T.process_wavelet(w, per)
    h, dt, nt = float(g['spacing']), float(g['dt']), int(g['nt'])
    e = [int(x) for x in g['extra']]
    ab = tuple(int(x) for x in g['absorbing'])
    f = npo.select_undersampling(wp[None], dt)
    vp_true = np.pad(g['vp_true'], [(e[0], e[0]), (e[1], e[1])], mode='edge')
    vp0 = np.full(vp_true.shape, 1500., np.float32)
    origin = (-e[0] * h, -e[1] * h)
    geo = T.geometry(g)
    inner = tuple(slice(a, s - a) for a, s in zip(e, vp_true.shape))
    win = npo.tukey(nt)
    worst = 0.

    def fwd(vp, wavelet, shot, save=False):
        return c_oracle.forward(vp, (h, h), dt, nt, ab, geo[[shot]], geo, wavelet[None], origin, kernel='OT2',
                                save=save, undersampling=f)

    def residual(obs, mod):
        obs_p = T.lowpass_cos(obs, per).astype(np.float32)
        mask = np.ones(obs_p.shape)
        mask[np.abs(obs_p) == 0.] = 0.
        mask = T.lowpass_cos(mask, per, zero_phase=True)
        m = T.lowpass_cos((mask * mod).astype(np.float32), per).astype(np.float32)
        o = T.lowpass_cos(obs_p, per).astype(np.float32)
        r = pipes.norm_per_shot(m) - pipes.norm_per_shot(o)
        return r, 0.5 * float(np.sum(np.asarray(r, np.float64) ** 2))

    grad = np.zeros(vp0.shape)
    prec = np.zeros(vp0.shape)
    for shot, recorded in zip(g['shot_ids'].tolist(), g['losses'].tolist()):
        mod, snaps = fwd(vp0, wp, shot, save=True)
        r, loss = residual(fwd(vp_true, w, shot)[0], mod)
        worst = max(worst, abs(loss / recorded - 1))
        print('iteration 1, shot %3d: recorded %.6f, oracle %.6f (%+.3f %%)' % (shot, recorded, loss,
                                                                               100 * (loss / recorded - 1)))
        adj = np.flip(T.lowpass_cos(np.flip(r, -1).astype(np.float32), per), -1).astype(np.float64) * win[None]
        late = np.zeros_like(adj)
        late[:, 2:] = adj[:, :-2]
        late[:, win > 0] /= win[None, win > 0]  # the oracle's adjoint applies the window itself
        gs, ps = c_oracle.adjoint(vp0, (h, h), dt, nt, ab, geo, np.ascontiguousarray(late.astype(np.float32)),
                                  origin, snaps, kernel='OT2', undersampling=f)
        grad += gs / vp0
        prec += ps / (vp0.astype(np.float64) ** 2)
    d, _ = pipes.apply_prec(grad[inner].astype(np.float32), prec[inner].astype(np.float32))
    d = d * pipes.field_mask(d.shape, (slice(None),) * d.ndim)
    d = pipes.smooth_field(d)
    d = pipes.norm_field(d, variable=vp0, transform=lambda x: 1 / x)
    vp1 = vp0.astype(np.float64)
    vp1[inner] = 1 / (1 / vp1[inner] - float(g['step_size']) * d)
    vp1 = np.clip(vp1, *g['clip']).astype(np.float32)
    for shot, recorded in zip(g['shot_ids2'].tolist(), g['losses2'].tolist()):
        _, loss = residual(fwd(vp_true, w, shot)[0], fwd(vp1, wp, shot)[0])
        worst = max(worst, abs(loss / recorded - 1))
        print('iteration 2, shot %3d: recorded %.6f, oracle %.6f (%+.3f %%)' % (shot, recorded, loss,
                                                                               100 * (loss / recorded - 1)))
    print('largest difference %.3f %%' % (100 * worst))
    return 0 if worst <= TOL else 1


if __name__ == '__main__':
    sys.exit(main())
