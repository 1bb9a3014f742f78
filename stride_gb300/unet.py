"""Learned FWI preconditioner: a 4-level U-Net trained and run with the project's own kernels.

The network maps [raw vp gradient, current vp] (two channels on the inner grid) to a vp update.
Every layer runs in libstrideacc.so: 3x3 convolutions are im2col + the tcgen05 BF16 GEMM
(``csrc/umma_gemm.cu``, FP32 accumulation in tensor memory) with bias and ReLU fused in its
epilogue; pooling, upsampling, concatenation, the backward passes, the MSE loss and Adam are the
kernels of ``csrc/unet_ops.cu``. Weights are FP32 masters packed to BF16 for the GEMMs.
Activations are NHWC FP32 tensors ([pixels][channels]); PyTorch only allocates them.

The reference has no learned component; this is the preconditioner of the inversion driver
``stride_gb300.fwi.LearnedFWI``.
"""

import ctypes

import numpy as np
import torch

from . import _lib, h5

__all__ = ['UNet', 'GraphTrainer']


def _up(x, m):
    return (x + m - 1) // m * m


def _s():
    return _lib._stream(torch.cuda.current_stream())


def _ck(rc):
    _lib.check(rc)


def _p(x):
    return _lib._ptr(x)


def _at(t, col):
    """Pointer to column `col` of the first row of a row-major tensor (channel slices)."""
    return ctypes.c_void_p(t.data_ptr() + col * t.element_size())


class _Conv:
    """k x k convolution (k = 3, padding 1, or k = 1) with bias and optional ReLU."""

    def __init__(self, cin, cout, relu, k, rng, dev):
        self.cin, self.cout, self.relu, self.k = cin, cout, relu, k
        self.kr = k * k * cin
        self.kp = _up(self.kr, 32)            # GEMM K (forward), N (input gradient)
        self.coutp = _up(cout, 32)            # GEMM N (forward), K (input gradient)
        self.mw = _up(self.coutp, 128)        # GEMM M (weight gradient)
        std = np.sqrt(2.0 / self.kr)          # He initialisation
        self.w = torch.as_tensor(rng.standard_normal((cout, self.kr)) * std, dtype=torch.float32, device=dev)
        self.b = torch.zeros(self.coutp, device=dev)
        self.gw = torch.zeros_like(self.w)
        self.gb = torch.zeros(self.coutp, device=dev)
        self.state = [torch.zeros_like(self.w), torch.zeros_like(self.w), torch.zeros_like(self.b),
                      torch.zeros_like(self.b)]
        self.wb = torch.empty((self.coutp, self.kp), dtype=torch.bfloat16, device=dev)
        self.wt = torch.empty((self.kp, self.coutp), dtype=torch.bfloat16, device=dev)
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        self.bscratch = torch.empty(128 * self.coutp, dtype=torch.float64, device=dev)  # bias-gradient parts
        self.pack()

    def params(self):
        return [(self.w, self.gw, self.state[0], self.state[1]), (self.b, self.gb, self.state[2], self.state[3])]

    def pack(self):
        _ck(_lib.load().sa_nn_pack_weights(_p(self.w), self.cout, self.kr, _p(self.wb), _p(self.wt), self.coutp,
                                           self.kp, _s()))

    def gemm(self, A, lda, B, ldb, C, ldc, M, N, K, bias=None, relu=False, accumulate=False, ksplit=1):
        _ck(_lib.load().sa_gemm_bf16(_p(A), lda, _p(B), ldb, _p(C), ldc, None, 0, M, N, K, _p(bias), int(relu),
                                     int(accumulate), ksplit, _p(self.err), _s()))

    def forward(self, x, B, H, W):
        lib = _lib.load()
        P = B * H * W
        y = torch.empty((P, self.coutp), device=x.device)
        if self.k == 3 and self.cin % 8 == 0:
            # implicit GEMM: the 3x3 neighbourhoods are gathered in shared memory from a bf16 copy of x
            xb = torch.empty((P, self.cin), dtype=torch.bfloat16, device=x.device)
            _ck(lib.sa_nn_to_bf16(_p(x), x.shape[1], P, self.cin, _p(xb), self.cin, _s()))
            _ck(lib.sa_conv3x3_bf16(_p(xb), self.cin, B, H, W, self.cin, _p(self.wb), self.kp, _p(y), self.coutp,
                                    None, 0, self.coutp, self.kp, _p(self.b), int(self.relu), _p(self.err), _s()))
            self.saved = (None, x, y, B, H, W)  # the weight gradient's im2col is built in backward
            return y
        col = torch.empty((P, self.kp), dtype=torch.bfloat16, device=x.device)
        if self.k == 3:
            _ck(lib.sa_nn_im2col(_p(x), x.shape[1], B, H, W, self.cin, _p(col), self.kp, _s()))
        else:
            col.zero_()
            _ck(lib.sa_nn_to_bf16(_p(x), x.shape[1], P, self.cin, _p(col), self.kp, _s()))
        self.gemm(col, self.kp, self.wb, self.kp, y, self.coutp, P, self.coutp, self.kp, bias=self.b, relu=self.relu)
        self.saved = (col, x, y, B, H, W)
        return y

    def backward(self, dy, need_dx=True):
        """dy [P][coutp] (modified in place by the ReLU backward); returns dx [P][cin] or None."""
        lib = _lib.load()
        col, x, y, B, H, W = self.saved
        P = B * H * W
        if col is None:
            col = torch.empty((P, self.kp), dtype=torch.bfloat16, device=dy.device)
            _ck(lib.sa_nn_im2col(_p(x), x.shape[1], B, H, W, self.cin, _p(col), self.kp, _s()))
        if self.relu:
            _ck(lib.sa_nn_relu_bwd(_p(dy), self.coutp, _p(y), self.coutp, P, self.coutp, _s()))
        _ck(lib.sa_nn_bias_grad(_p(dy), self.coutp, P, self.coutp, _p(self.gb), _p(self.bscratch), _s()))
        dyb = torch.empty((P, self.coutp), dtype=torch.bfloat16, device=dy.device)
        _ck(lib.sa_nn_to_bf16(_p(dy), self.coutp, P, self.coutp, _p(dyb), self.coutp, _s()))
        # weight gradient: dW[mw][kp] = dy^T col (K = pixels, split over CTAs)
        dyT = torch.empty((self.mw, P), dtype=torch.bfloat16, device=dy.device)
        _ck(lib.sa_nn_transpose_bf16(_p(dyb), self.coutp, P, self.coutp, _p(dyT), P, self.mw, _s()))
        colT = torch.empty((self.kp, P), dtype=torch.bfloat16, device=dy.device)
        _ck(lib.sa_nn_transpose_bf16(_p(col), self.kp, P, self.kp, _p(colT), P, self.kp, _s()))
        # split K over the pixels: each split stores its partial product to its own slab, summed in a
        # fixed order (reproducible training)
        ksplit = max(1, min(64, P // 2048))
        dw = torch.zeros((self.mw, self.kp), device=dy.device)
        if ksplit > 1:
            nk = -(-P // 64)
            per = -(-nk // ksplit)
            nz = -(-nk // per)  # splits the GEMM launches
            slabs = torch.empty((nz, self.mw, self.kp), device=dy.device)
            self.gemm(dyT, P, colT, P, slabs, self.kp, self.mw, self.kp, P, accumulate=2, ksplit=ksplit)
            _ck(lib.sa_nn_sum_slabs(_p(slabs), self.mw * self.kp, nz, _p(dw), self.mw * self.kp, 0, _s()))
        else:
            self.gemm(dyT, P, colT, P, dw, self.kp, self.mw, self.kp, P, accumulate=True)
        self.gw.copy_(dw[:self.cout, :self.kr])
        if not need_dx:
            return None
        # input gradient: dcol[P][kp] = dy wt^T, then col2im
        dcol = torch.empty((P, self.kp), device=dy.device)
        self.gemm(dyb, self.coutp, self.wt, self.coutp, dcol, self.kp, P, self.kp, self.coutp)
        dx = torch.empty((P, self.cin), device=dy.device)
        if self.k == 3:
            _ck(lib.sa_nn_col2im(_p(dcol), self.kp, B, H, W, self.cin, _p(dx), self.cin, 0, _s()))
        else:
            _ck(lib.sa_nn_copy_channels(_p(dcol), self.kp, P, self.cin, _p(dx), self.cin, 0, _s()))
        return dx


class UNet:
    """4-level U-Net (base channels 32: 32-64-128-256), two 3x3 conv + ReLU per level, 2x2 max
    pooling, nearest upsampling + 3x3 conv, skip concatenation, 1x1 output conv."""

    def __init__(self, cin=2, cout=1, base=32, levels=4, seed=0, device=None):
        dev = torch.device(device) if device is not None else torch.device('cuda', torch.cuda.current_device())
        rng = np.random.default_rng(seed)
        self.levels = levels
        self.ch = [base * 2 ** l for l in range(levels)]
        ch = self.ch
        self.enc = []
        for l in range(levels):
            cin_l = cin if l == 0 else ch[l - 1]
            self.enc.append((_Conv(cin_l, ch[l], True, 3, rng, dev), _Conv(ch[l], ch[l], True, 3, rng, dev)))
        self.up = [_Conv(ch[l + 1], ch[l], True, 3, rng, dev) for l in range(levels - 1)]
        self.dec = [(_Conv(2 * ch[l], ch[l], True, 3, rng, dev), _Conv(ch[l], ch[l], True, 3, rng, dev))
                    for l in range(levels - 1)]
        self.out = _Conv(ch[0], cout, False, 1, rng, dev)
        self.cout = cout
        self.step_count = 0
        self.device = dev

    def layers(self):
        ls = [c for pair in self.enc for c in pair] + self.up + [c for pair in self.dec for c in pair] + [self.out]
        return ls

    def forward(self, x):
        """x: [B, H, W, cin] float32 CUDA (H, W divisible by 2^(levels-1), B*H*W / 4^(levels-1) a
        multiple of 128); returns the padded [B*H*W][coutp] result (``output`` extracts the image)."""
        lib = _lib.load()
        B, H, W, _ = x.shape
        a = x.reshape(B * H * W, -1).contiguous()
        self.shapes = []
        self.skips = []
        self.pool_in = []
        h, w = H, W
        for l in range(self.levels):
            a = self.enc[l][0].forward(a, B, h, w)
            a = self.enc[l][1].forward(a, B, h, w)
            self.shapes.append((h, w))
            if l < self.levels - 1:
                self.skips.append(a)
                p = torch.empty((B * (h // 2) * (w // 2), self.ch[l]), device=x.device)
                _ck(lib.sa_nn_maxpool(_p(a), self.ch[l], B, h, w, self.ch[l], _p(p), self.ch[l], _s()))
                self.pool_in.append(a)
                a = p
                h, w = h // 2, w // 2
        for l in reversed(range(self.levels - 1)):
            h, w = self.shapes[l]
            c = self.ch[l]
            u = torch.empty((B * h * w, self.ch[l + 1]), device=x.device)
            _ck(lib.sa_nn_upsample(_p(a), self.ch[l + 1], B, h, w, self.ch[l + 1], _p(u), self.ch[l + 1], _s()))
            u = self.up[l].forward(u, B, h, w)
            cat = torch.empty((B * h * w, 2 * c), device=x.device)
            _ck(lib.sa_nn_copy_channels(_p(u), c, B * h * w, c, _p(cat), 2 * c, 0, _s()))
            _ck(lib.sa_nn_copy_channels(_p(self.skips[l]), c, B * h * w, c, _at(cat, c), 2 * c, 0, _s()))
            a = self.dec[l][0].forward(cat, B, h, w)
            a = self.dec[l][1].forward(a, B, h, w)
        y = self.out.forward(a, B, H, W)
        self.B = B
        return y  # [B*H*W][coutp]: channels 0..cout-1 are the output

    def output(self, y, B, H, W):
        """The [B, H, W, cout] output of the padded result of forward()."""
        lib = _lib.load()
        o = torch.empty((B * H * W, self.cout), device=y.device)
        _ck(lib.sa_nn_copy_channels(_p(y), self.out.coutp, B * H * W, self.cout, _p(o), self.cout, 0, _s()))
        return o.reshape(B, H, W, self.cout)

    def backward(self, d):
        """d [B*H*W][coutp] (gradient of forward()'s result, zero beyond cout; overwritten): sets every
        layer's gradients."""
        lib = _lib.load()
        B = self.B
        da = self.out.backward(d)
        dskips = [None] * (self.levels - 1)
        for l in range(self.levels - 1):
            h, w = self.shapes[l]
            c = self.ch[l]
            da = self.dec[l][1].backward(da)
            dcat = self.dec[l][0].backward(da)
            du = torch.empty((B * h * w, c), device=dcat.device)
            _ck(lib.sa_nn_copy_channels(_p(dcat), 2 * c, B * h * w, c, _p(du), c, 0, _s()))
            dskips[l] = torch.empty((B * h * w, c), device=dcat.device)
            _ck(lib.sa_nn_copy_channels(_at(dcat, c), 2 * c, B * h * w, c, _p(dskips[l]), c, 0, _s()))
            dup = self.up[l].backward(du)  # gradient of the upsampled input [B*h*w][ch[l+1]]
            hn, wn = self.shapes[l + 1]
            da = torch.empty((B * hn * wn, self.ch[l + 1]), device=d.device)
            _ck(lib.sa_nn_upsample_bwd(_p(dup), self.ch[l + 1], B, h, w, self.ch[l + 1], _p(da), self.ch[l + 1], _s()))
        for l in reversed(range(self.levels)):
            h, w = self.shapes[l]
            if l < self.levels - 1:  # output of level l fed the pool (gradient da of level l+1's input) and the skip
                g = dskips[l]
                _ck(lib.sa_nn_maxpool_bwd(_p(self.pool_in[l]), self.ch[l], _p(da), self.ch[l], B, h, w, self.ch[l],
                                          _p(g), self.ch[l], 1, _s()))
                da = g
            da = self.enc[l][1].backward(da)
            da = self.enc[l][0].backward(da, need_dx=False) if l == 0 else self.enc[l][0].backward(da)

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        lib = _lib.load()
        self.step_count += 1
        for layer in self.layers():
            for w, g, m, v in layer.params():
                _ck(lib.sa_nn_adam(_p(w), _p(g), _p(m), _p(v), w.numel(), lr, b1, b2, eps, self.step_count, _s()))
            layer.pack()

    def adam_step_dev(self, lr, b1, b2, eps, c12, nsteps, step):
        """adam_step with the step count in device memory (a captured training step)."""
        lib = _lib.load()
        for layer in self.layers():
            for w, g, m, v in layer.params():
                _ck(lib.sa_nn_adam_dev(_p(w), _p(g), _p(m), _p(v), w.numel(), lr, b1, b2, eps, _p(c12), nsteps,
                                       _p(step), _s()))
            layer.pack()

    def mse(self, y, target):
        """Mean squared error of channel 0 of forward()'s result y against target [B, H, W] and its
        gradient, shaped for backward()."""
        lib = _lib.load()
        t = target.contiguous()
        d = torch.zeros_like(y)
        loss = torch.zeros(1, dtype=torch.float64, device=y.device)
        _ck(lib.sa_nn_mse(_p(y), self.out.coutp, _p(t), t.numel(), _p(d), self.out.coutp, _p(loss), _s()))
        return loss, d

    def errors(self):
        return sum(int(layer.err.item()) for layer in self.layers())

    def state_dict(self):
        return {'%d_%s' % (i, n): t.detach().cpu().numpy() for i, layer in enumerate(self.layers())
                for n, t in (('w', layer.w), ('b', layer.b))}

    def load_state_dict(self, sd):
        for i, layer in enumerate(self.layers()):
            layer.w.copy_(torch.as_tensor(sd['%d_w' % i]))
            layer.b.copy_(torch.as_tensor(sd['%d_b' % i]))
            layer.pack()

    def dump(self, filename):
        """The weights as an HDF5 file: one dataset per layer weight and bias (state_dict names)."""
        h5.write_file(filename, self.state_dict())

    def load(self, filename):
        """Weights from a file written by ``dump``."""
        self.load_state_dict(h5.HDF5(filename, mode='r').load(lazy=False))


class GraphTrainer:
    """One Adam step of a UNet on batches of a fixed shape (forward, MSE, backward, Adam, BF16
    repack) captured once as a CUDA graph and replayed per batch: one launch instead of the
    step's few hundred kernel calls from the host. The step count lives in device memory and the
    bias corrections in a table formed as adam_step forms them, so a replayed step is bit for bit
    the eager step. The loss is summed on the device (loss_sum)."""

    def __init__(self, net, B, H, W, cin, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, max_steps=1 << 16):
        lib = _lib.load()
        dev = net.device
        self.net = net
        self.x = torch.zeros((B, H, W, cin), device=dev)
        self.t = torch.zeros((B, H, W), device=dev)
        self.step = torch.full((1,), net.step_count, dtype=torch.int32, device=dev)
        self.max_steps = max_steps
        self.c12 = torch.empty(2 * max_steps, device=dev)
        _ck(lib.sa_nn_adam_corrections(b1, b2, max_steps, _p(self.c12)))
        self.loss_sum = torch.zeros(1, dtype=torch.float64, device=dev)
        # warm-up on a side stream: kernel attributes set, no weight updated
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            y = net.forward(self.x)
            _, d = net.mse(y, self.t)
            net.backward(d)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            y = net.forward(self.x)
            loss, d = net.mse(y, self.t)
            net.backward(d)
            self.step += 1
            net.adam_step_dev(lr, b1, b2, eps, self.c12, max_steps, self.step)
            self.loss_sum += loss

    def train_step(self, x, t):
        """One step on the batch x [B, H, W, cin], target t [B, H, W]."""
        self.x.copy_(x)
        self.t.copy_(t)
        self.graph.replay()
        self.net.step_count += 1

