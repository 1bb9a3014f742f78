"""L2 trace misfit (stride/optimisation/loss/l2_distance.py:13-68)."""

import numpy as np

__all__ = ['L2DistanceLoss']


class L2DistanceLoss:
    """f = 1/2 ||modelled - observed||^2; the adjoint source for ``modelled`` is the residual
    (modelled - observed) scaled by the incoming gradient."""

    def __init__(self, **kwargs):
        self.residual = None

    def forward(self, modelled, observed, **kwargs):
        m = getattr(modelled, 'data', modelled)
        o = getattr(observed, 'data', observed)
        self.residual = np.asarray(m, dtype=np.float32) - np.asarray(o, dtype=np.float32)
        return 0.5 * float(np.sum(self.residual.astype(np.float64) ** 2))

    __call__ = forward

    def adjoint(self, d_fun=1.0, modelled=None, observed=None, **kwargs):
        r = self.residual
        self.residual = None
        return np.float32(d_fun) * r, -np.float32(d_fun) * r
