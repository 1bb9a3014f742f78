"""PyTorch autograd around the batched forward map vp -> traces (2D and 3D).

``WaveOperator`` binds one plan (grid, time axis, physics options, geometry of all shots and
their wavelets); ``op(vp)`` returns the traces of every shot as a CUDA tensor whose backward
is the hand-written exact adjoint of the discrete forward map (``SA_GRAD_EXACT``): the forward
keeps checkpoints of the wavefield every ``checkpoint_interval`` steps and the backward
recomputes each segment from them. The gradient is dL/dvp on the extended grid, so it agrees
with central finite differences of the forward itself; the reference's imaging-condition
gradient (``IsoAcousticGB300.get_grad_vp``) remains the Stride-facing path.

In the reference the same role is played by Stride's operator graph: ``Operator.__call__`` /
``__call_adjoint__`` (stride/core.py:728-825) chaining ``IsoAcousticDevito`` forward and
adjoint (stride/physics/iso_acoustic/devito.py:220-1113).
"""

import numpy as np
import torch

from . import _lib

__all__ = ['WaveOperator']


class _ForwardMap(torch.autograd.Function):

    @staticmethod
    def forward(ctx, vp, op):
        traces = op._run_forward(vp)
        ctx.op = op
        ctx.token = op._token
        ctx.save_for_backward(vp)
        return traces

    @staticmethod
    def backward(ctx, grad_traces):
        op = ctx.op
        (vp,) = ctx.saved_tensors
        if op._token != ctx.token:  # another forward ran since: rebuild this one's checkpoints
            op._run_forward(vp)
        return op._run_adjoint(grad_traces), None


class WaveOperator:
    """Forward map of a batch of 2D or 3D shots on one GPU, differentiable in vp.

    shape/spacing/extra/absorbing describe the extended grid as the plan does; src_offsets /
    rec_offsets are CSR offsets of each shot's points, src_xyz / rec_xyz their coordinates
    (inner-domain frame, metres); wavelets [n_src, nt] are the source samples (windowed as the
    reference stores them). rho and alpha (dB/cm) are fixed (not differentiated).
    """

    def __init__(self, shape, spacing, extra, absorbing, dt, nt, src_offsets, src_xyz, rec_offsets, rec_xyz,
                 wavelets, rho=None, alpha=None, kernel='OT4', checkpoint_interval=50, checkpoint_budget=0.0,
                 device=None):
        self.device = torch.device(device) if device is not None else torch.device('cuda', torch.cuda.current_device())
        n_shots = len(src_offsets) - 1
        if rho is None:
            density = _lib.SA_DENSITY_NONE
        else:
            r = np.asarray(rho, np.float32)
            density = _lib.SA_DENSITY_CONSTANT if np.isclose(r.min(), r.max()) else _lib.SA_DENSITY_VARIABLE
        with torch.cuda.device(self.device):
            self.plan = _lib.Plan(len(shape), shape, spacing, extra, absorbing, dt, nt, kernel=kernel, density=density,
                                  attenuation=alpha is not None, undersampling=1, max_shots=n_shots,
                                  checkpoint_interval=checkpoint_interval, checkpoint_budget=checkpoint_budget)
        self.shape = tuple(int(s) for s in shape)
        self.nt = int(nt)
        self._rho = None if rho is None else torch.as_tensor(np.ascontiguousarray(rho, np.float32), device=self.device)
        self._alpha = None if alpha is None else torch.as_tensor(np.ascontiguousarray(alpha, np.float32),
                                                                 device=self.device)
        self._geometry = (np.asarray(src_offsets), np.asarray(src_xyz, np.float32), np.asarray(rec_offsets),
                          np.asarray(rec_xyz, np.float32))
        self._geometry_set = False
        self.wavelets = torch.as_tensor(np.ascontiguousarray(wavelets, np.float32), device=self.device)
        self._token = 0

    @property
    def n_rec(self):
        return int(self._geometry[2][-1])

    def _set_medium(self, vp):
        vp = vp.detach().to(self.device, torch.float32).contiguous()
        if tuple(vp.shape) != self.shape:
            raise ValueError('vp has shape %s, the plan %s' % (tuple(vp.shape), self.shape))
        torch.cuda.current_stream(self.device).synchronize()
        self.plan.set_medium(vp, self._rho, self._alpha)
        if not self._geometry_set:
            self.plan.set_geometry(*self._geometry)
            self._geometry_set = True

    def _run_forward(self, vp):
        with torch.cuda.device(self.device):
            self._set_medium(vp)
            traces = torch.empty((self.n_rec, self.nt), device=self.device)
            self.plan.forward(self.wavelets, traces, save='checkpoints', stream=torch.cuda.current_stream())
            self._token += 1
            return traces

    def _run_adjoint(self, grad_traces):
        with torch.cuda.device(self.device):
            g = torch.empty(self.shape, device=self.device)
            p = torch.empty(self.shape, device=self.device)
            self.plan.adjoint(grad_traces.detach().to(self.device, torch.float32).contiguous(), g, p,
                              stream=torch.cuda.current_stream(), exact=True)
            return g

    def __call__(self, vp):
        """Traces [n_rec_total, nt] of every shot for the velocity vp (extended grid)."""
        return _ForwardMap.apply(vp, self)

    def close(self):
        self.plan.close()
