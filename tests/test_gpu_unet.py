"""Learned preconditioner kernels: the tcgen05 BF16 GEMM against an FP64 product of the same
bf16 operands."""

import pytest

torch = pytest.importorskip('torch')

from stride_gb300 import _lib  # noqa: E402

pytestmark = pytest.mark.gpu


def _gemm(A, B, C=None, bias=None, relu=False, accumulate=False, want_bf16=False, ksplit=1):
    M, K = A.shape
    N = B.shape[0]
    C = torch.zeros((M, N), device='cuda') if C is None else C
    Cb = torch.zeros((M, N), dtype=torch.bfloat16, device='cuda') if want_bf16 else None
    err = torch.zeros(1, dtype=torch.int32, device='cuda')
    _lib.check(_lib.load().sa_gemm_bf16(_lib._ptr(A), A.stride(0), _lib._ptr(B), B.stride(0), _lib._ptr(C), C.stride(0),
                                        _lib._ptr(Cb), N, M, N, K, _lib._ptr(bias), int(relu), int(accumulate), ksplit,
                                        _lib._ptr(err), _lib._stream(torch.cuda.current_stream())))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return C, Cb


@pytest.mark.parametrize("M,N,K", [(128, 32, 64), (256, 64, 128), (384, 128, 192), (128, 256, 64), (256, 96, 320),
                                   (128, 64, 32), (256, 32, 80), (128, 128, 288)])
def test_gemm_bf16(M, N, K):
    g = torch.Generator(device='cpu').manual_seed(M + N + K)
    A = torch.randn((M, K), generator=g).to(torch.bfloat16).cuda()
    B = torch.randn((N, K), generator=g).to(torch.bfloat16).cuda()
    C, _ = _gemm(A, B)
    ref = A.double() @ B.double().T
    err = float((C.double() - ref).norm() / ref.norm())
    assert err <= 1e-5, err


def test_gemm_epilogue():
    g = torch.Generator(device='cpu').manual_seed(7)
    M, N, K = 256, 64, 128
    A = torch.randn((M, K), generator=g).to(torch.bfloat16).cuda()
    B = torch.randn((N, K), generator=g).to(torch.bfloat16).cuda()
    C0 = torch.randn((M, N), generator=g).cuda()
    bias = torch.randn(N, generator=g).cuda()
    C, Cb = _gemm(A, B, C=C0.clone(), bias=bias, relu=True, accumulate=True, want_bf16=True)
    ref = torch.relu(C0.double() + A.double() @ B.double().T + bias.double())
    assert float((C.double() - ref).norm() / ref.norm()) <= 1e-5
    assert torch.equal(Cb, C.to(torch.bfloat16))


def test_gemm_split_k():
    g = torch.Generator(device='cpu').manual_seed(3)
    M, N, K = 128, 64, 64 * 37 + 32
    A = torch.randn((M, K), generator=g).to(torch.bfloat16).cuda()
    B = torch.randn((N, K), generator=g).to(torch.bfloat16).cuda()
    C0 = torch.randn((M, N), generator=g).cuda()
    C, _ = _gemm(A, B, C=C0.clone(), accumulate=True, ksplit=5)
    ref = C0.double() + A.double() @ B.double().T
    assert float((C.double() - ref).norm() / ref.norm()) <= 1e-5


@pytest.mark.parametrize("B,H,W,Cin,N", [(2, 16, 8, 8, 32), (1, 16, 16, 32, 64), (2, 8, 24, 64, 128),
                                         (1, 32, 4, 16, 32)])
def test_conv3x3_implicit_gemm(B, H, W, Cin, N):
    """The implicit-GEMM 3x3 convolution (neighbourhoods gathered in shared memory, zero padding at
    the image edges, columns (ky*3+kx)*Cin+ci) against an FP64 convolution of the same bf16 values,
    with bias and ReLU."""
    g = torch.Generator(device='cpu').manual_seed(B * 1000 + H * 10 + Cin)
    x = torch.randn((B, H, W, Cin), generator=g).to(torch.bfloat16)
    K = 9 * Cin
    Kp = (K + 31) // 32 * 32
    w = torch.randn((N, 3, 3, Cin), generator=g).to(torch.bfloat16)  # [N][ky][kx][ci]
    Wt = torch.zeros((N, Kp), dtype=torch.bfloat16)
    Wt[:, :K] = w.reshape(N, K)
    bias = torch.randn(N, generator=g)
    P = B * H * W
    C = torch.zeros((P, N), device='cuda')
    err = torch.zeros(1, dtype=torch.int32, device='cuda')
    xd, Wd, bd = x.reshape(P, Cin).contiguous().cuda(), Wt.cuda(), bias.cuda()
    _lib.check(_lib.load().sa_conv3x3_bf16(_lib._ptr(xd), Cin, B, H, W, Cin, _lib._ptr(Wd), Kp, _lib._ptr(C), N,
                                           None, 0, N, Kp, _lib._ptr(bd), 1, _lib._ptr(err),
                                           _lib._stream(torch.cuda.current_stream())))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = torch.nn.functional.conv2d(x.double().permute(0, 3, 1, 2), w.double().permute(0, 3, 1, 2),
                                     bias.double(), padding=1).permute(0, 2, 3, 1).reshape(P, N).relu()
    rel = float((C.cpu().double() - ref).norm() / ref.norm())
    assert rel <= 1e-5, rel


def test_gemm_split_k_slabs_are_reproducible():
    """Split K into slabs (accumulate 2) and their fixed-order sum: the product, bit for bit the same
    on every run."""
    g = torch.Generator(device='cpu').manual_seed(4)
    M, N, K = 256, 64, 64 * 37 + 32
    A = torch.randn((M, K), generator=g).to(torch.bfloat16).cuda()
    B = torch.randn((N, K), generator=g).to(torch.bfloat16).cuda()
    nk = -(-K // 64)
    per = -(-nk // 5)
    nz = -(-nk // per)
    outs = []
    for _ in range(3):
        slabs = torch.full((nz, M, N), float('nan'), device='cuda')  # every slab element is written
        _gemm(A, B, C=slabs[0], accumulate=2, ksplit=5)
        out = torch.empty((M, N), device='cuda')
        _lib.check(_lib.load().sa_nn_sum_slabs(_lib._ptr(slabs), M * N, nz, _lib._ptr(out), M * N, 0,
                                               _lib._stream(torch.cuda.current_stream())))
        torch.cuda.synchronize()
        outs.append(out)
    ref = A.double() @ B.double().T
    assert float((outs[0].double() - ref).norm() / ref.norm()) <= 1e-5
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[0], outs[2])


def _reference_net(net, x, target):
    """The same U-Net in float64 PyTorch on the CPU (weights as the BF16 the GEMMs use)."""
    F = torch.nn.functional

    def conv(layer, a):
        w = layer.w.detach().cpu().to(torch.bfloat16).double()
        k = layer.k
        w = w.reshape(layer.cout, k, k, layer.cin).permute(0, 3, 1, 2).contiguous().requires_grad_(True)
        b = layer.b.detach().cpu()[:layer.cout].double().requires_grad_(True)
        y = F.conv2d(a, w, b, padding=k // 2)
        return (F.relu(y) if layer.relu else y), w, b

    params = []
    a = x.permute(0, 3, 1, 2).double()
    skips = []
    for l in range(net.levels):
        for layer in net.enc[l]:
            a, w, b = conv(layer, a)
            params.append((layer, w, b))
        if l < net.levels - 1:
            skips.append(a)
            a = F.max_pool2d(a, 2)
    for l in reversed(range(net.levels - 1)):
        u = F.interpolate(a, scale_factor=2, mode='nearest')
        u, w, b = conv(net.up[l], u)
        params.append((net.up[l], w, b))
        a = torch.cat([u, skips[l]], dim=1)
        for layer in net.dec[l]:
            a, w, b = conv(layer, a)
            params.append((layer, w, b))
    out, w, b = conv(net.out, a)
    params.append((net.out, w, b))
    loss = ((out[:, 0] - target.double()) ** 2).mean()
    loss.backward()
    return out[:, 0].detach(), loss.item(), params


def test_unet_forward_backward_against_torch():
    """Output and loss within 2 % and every layer's weight and bias gradient with cosine >= 0.99
    against an FP64 reference: the GEMM operands (activations, weights, back-propagated
    gradients) are BF16, whose rounding accumulates over the 23 layers of the backward pass."""
    from stride_gb300.unet import UNet
    torch.manual_seed(0)
    B, H, W = 2, 64, 64
    net = UNet(seed=1)
    x = torch.randn(B, H, W, 2)
    target = torch.randn(B, H, W)
    y = net.forward(x.cuda())
    loss, d = net.mse(y, target.cuda())
    net.backward(d)
    torch.cuda.synchronize()
    assert net.errors() == 0
    out = net.output(y, B, H, W)[..., 0].cpu().double()
    ref_out, ref_loss, params = _reference_net(net, x, target)
    assert float((out - ref_out).norm() / ref_out.norm()) <= 2e-2
    assert abs(float(loss.item()) - ref_loss) <= 2e-2 * ref_loss
    for layer, w, b in params:
        g = layer.gw.cpu().double().reshape(layer.cout, layer.k, layer.k, layer.cin).permute(0, 3, 1, 2)
        cos = float((g * w.grad).sum() / (g.norm() * w.grad.norm() + 1e-30))
        assert cos >= 0.99, (layer.cin, layer.cout, cos)
        gb = layer.gb.cpu().double()[:layer.cout]
        cosb = float((gb * b.grad).sum() / (gb.norm() * b.grad.norm() + 1e-30))
        assert cosb >= 0.99, (layer.cin, layer.cout, cosb)


def test_unet_training_reduces_loss():
    from stride_gb300.unet import UNet
    torch.manual_seed(1)
    B, H, W = 4, 64, 64
    net = UNet(seed=2)
    x = torch.randn(B, H, W, 2, device='cuda')
    yy, xx = torch.meshgrid(torch.linspace(-1, 1, H), torch.linspace(-1, 1, W), indexing='ij')
    target = (x[..., 0] * 0.5 + torch.exp(-(yy ** 2 + xx ** 2) * 4).cuda()).contiguous()
    losses = []
    for _ in range(60):
        y = net.forward(x)
        loss, d = net.mse(y, target)
        net.backward(d)
        net.adam_step(lr=1e-3)
        losses.append(float(loss.item()))
    assert net.errors() == 0
    assert losses[-1] < 0.3 * losses[0], losses[::10]


def test_unet_training_is_reproducible():
    """Training is deterministic (split-K slabs summed in a fixed order, fixed-order bias sums):
    two networks from the same seed, trained on the same batches, end bit for bit equal."""
    from stride_gb300.unet import UNet
    torch.manual_seed(3)
    B, H, W = 4, 64, 64
    x = torch.randn(B, H, W, 2, device='cuda')
    target = torch.randn(B, H, W, device='cuda')
    nets = []
    for _ in range(2):
        net = UNet(seed=5)
        for _ in range(8):
            y = net.forward(x)
            _, d = net.mse(y, target)
            net.backward(d)
            net.adam_step(lr=1e-3)
        nets.append(net)
    for (a, _, _, _), (b, _, _, _) in zip((p for l in nets[0].layers() for p in l.params()),
                                          (p for l in nets[1].layers() for p in l.params())):
        assert torch.equal(a, b)



def test_graph_training_step_equals_eager():
    """A training step captured as a CUDA graph and replayed (unet.GraphTrainer) leaves the network
    bit for bit where the eager steps do."""
    from stride_gb300.unet import GraphTrainer, UNet
    torch.manual_seed(4)
    B, H, W = 4, 64, 64
    xs = [torch.randn(B, H, W, 2, device='cuda') for _ in range(5)]
    ts = [torch.randn(B, H, W, device='cuda') for _ in range(5)]
    eager = UNet(seed=7)
    loss_eager = 0.0
    for x, t in zip(xs, ts):
        y = eager.forward(x)
        loss, d = eager.mse(y, t)
        eager.backward(d)
        eager.adam_step(lr=1e-3)
        loss_eager += float(loss.item())
    graphed = UNet(seed=7)
    trainer = GraphTrainer(graphed, B, H, W, 2, lr=1e-3)
    for x, t in zip(xs, ts):
        trainer.train_step(x, t)
    # the loss is an FP64 sum whose atomic accumulation order varies: equal to rounding
    assert abs(float(trainer.loss_sum.item()) - loss_eager) <= 1e-12 * abs(loss_eager)
    assert eager.errors() == 0 and graphed.errors() == 0
    for la, lb in zip(eager.layers(), graphed.layers()):
        for (a, _, _, _), (b, _, _, _) in zip(la.params(), lb.params()):
            assert torch.equal(a, b)
