"""U-Net preconditioner kernels against PyTorch CPU autograd (float32) on the
same weights; the reference rounds weights, the network input and every
hidden activation to bf16 like the GPU path, so the remaining differences
are the bf16 rounding of the backward operands."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _bf(x):
    return x.to(torch.bfloat16).to(torch.float32)


def ref_forward(net, weights, x):
    """Same topology as pylops_gb300.learned.UNet, NCHW, torch CPU."""
    import torch.nn.functional as F

    scale = 1.0 / torch.sqrt(torch.mean(x.double() ** 2, dim=(1, 2))).float()
    h = _bf(x * scale[:, None, None])[:, None]

    def conv(i, inp):
        c = net.convs[i]
        w, b = weights[i]
        y = F.conv2d(inp, _bf(w), b, stride=c.stride, padding=c.ks // 2)
        if c.relu:
            y = torch.relu(y)
        return _bf(y) if i != net.head else y

    skips = []
    for l, (a, b) in enumerate(net.enc):
        h = conv(b, conv(a, h))
        skips.append(h)
    for l in range(net.levels - 2, -1, -1):
        a, b = net.dec[l]
        up = h.repeat_interleave(2, dim=2).repeat_interleave(2, dim=3)
        h = conv(b, conv(a, torch.cat([up, skips[l]], dim=1)))
    return conv(net.head, h)[:, 0]


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.mark.parametrize("levels,base,B,H,W", [(3, 8, 2, 16, 32), (4, 16, 1, 32, 16), (4, 16, 1, 64, 256)])
def test_unet_forward_and_gradients_match_cpu_autograd(levels, base, B, H, W):
    from pylops_gb300.learned.unet import UNet

    net = UNet(levels=levels, base=base, seed=3)
    g = torch.Generator().manual_seed(5)
    x = torch.randn(B, H, W, generator=g)
    t = 0.5 * torch.randn(B, H, W, generator=g)
    out = net.forward(x.cuda()).cpu()
    loss = float(net.loss_and_grad(x.cuda(), t.cuda()))
    grads = net.gradients()
    net.check_errors()

    ws = [(torch.tensor(w, requires_grad=True), torch.tensor(b, requires_grad=True)) for w, b in net.get_weights()]
    ref = ref_forward(net, ws, x)
    ref_loss = torch.mean((ref - t) ** 2)
    ref_loss.backward()
    assert _rel(out.numpy(), ref.detach().numpy()) < 1e-2
    assert abs(loss - float(ref_loss)) / float(ref_loss) < 1e-2
    for i, ((gw, gb), (w, b)) in enumerate(zip(grads, ws)):
        ew = _rel(gw, w.grad.numpy())
        eb = _rel(gb, b.grad.numpy())
        assert ew < 5e-2, f"layer {i} weight gradient error {ew:.3e}"
        assert eb < 5e-2, f"layer {i} bias gradient error {eb:.3e}"


def test_unet_training_is_deterministic_and_lowers_the_loss():
    from pylops_gb300.learned.unet import UNet

    g = torch.Generator().manual_seed(11)
    x = torch.randn(4, 32, 32, generator=g).cuda()
    t = torch.relu(x)  # a pointwise map of the input: learnable
    a, b = UNet(levels=3, base=8, seed=0), UNet(levels=3, base=8, seed=0)
    losses = []
    for _ in range(60):
        la = float(a.train_step(x, t, lr=3e-3))
        lb = float(b.train_step(x, t, lr=3e-3))
        assert la == lb
        losses.append(la)
    assert torch.equal(a.params, b.params)
    assert losses[-1] < 0.3 * losses[0], losses[::10]
    a.check_errors()


def test_splitk_gemm_matches_fp32_reference():
    from pylops_gb300 import _native

    g = torch.Generator().manual_seed(2)
    for M, N, K, splits in [(32, 288, 4096, 0), (1, 32, 2048, 7), (64, 9, 1024, 3), (128, 200, 520, 1)]:
        A = torch.randn(M, K, generator=g).to(torch.bfloat16)
        B = torch.randn(N, K, generator=g).to(torch.bfloat16)
        ldc = N + 8
        C = torch.full((M, ldc), 7.0, device="cuda")
        work = torch.empty(1 << 20, device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        Ad, Bd = A.cuda(), B.cuda()
        _native.check(_native.lib().kgb_gemm_bf16_tn_splitk(
            Ad.data_ptr(), Bd.data_ptr(), C.data_ptr(), M, N, K, K, K, ldc, splits, work.data_ptr(), work.numel(),
            err.data_ptr(), torch.cuda.current_stream().cuda_stream))
        ref = A.float() @ B.float().T
        got = C.cpu()
        assert int(err.item()) == 0
        assert _rel(got[:, :N].numpy(), ref.numpy()) < 1e-5
        assert torch.all(got[:, N:] == 7.0)


@pytest.mark.parametrize("B,H,W,C,N,flip", [(2, 16, 32, 32, 32, 0), (1, 8, 256, 96, 64, 0), (2, 32, 64, 64, 96, 1),
                                            (1, 64, 128, 40, 128, 1), (2, 6, 256, 32, 32, 1),
                                            (3, 2, 128, 128, 64, 0), (2, 8, 64, 64, 192, 1), (1, 4, 32, 128, 256, 0),
                                            (1, 8, 64, 64, 320, 0), (2, 2, 128, 64, 144, 1)])
def test_implicit_conv3x3_matches_conv2d(B, H, W, C, N, flip):
    """kgb_conv3x3_bf16 (4-D TMA boxes shifted per tap, zero fill as padding;
    for W a multiple of 128 one halo row per ky shared by the three kx taps)
    against torch conv2d on the same bf16-rounded operands; flip = 1 is the
    transposed convolution (kernel flipped in both axes)."""
    import torch.nn.functional as F

    from pylops_gb300 import _native

    g = torch.Generator().manual_seed(B * 1000 + C + N)
    x = _bf(torch.randn(B, H, W, C, generator=g))
    w = _bf(torch.randn(N, C, 3, 3, generator=g) / (3 * C ** 0.5))
    bias = torch.randn(N, generator=g)
    Cp = (C + 63) // 64 * 64
    wi = torch.zeros(N, 9, Cp)
    wi[:, :, :C] = w.permute(0, 2, 3, 1).reshape(N, 9, C)
    xd = x.to(torch.bfloat16).cuda().contiguous()
    wd = wi.reshape(N, 9 * Cp).to(torch.bfloat16).cuda().contiguous()
    y = torch.empty(B * H * W, N, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    bd = bias.cuda()
    _native.check(_native.lib().kgb_conv3x3_bf16(xd.data_ptr(), wd.data_ptr(), y.data_ptr(), B, H, W, C, N, flip,
                                                 None if flip else bd.data_ptr(), 0, err.data_ptr(),
                                                 torch.cuda.current_stream().cuda_stream))
    ref = F.conv2d(x.permute(0, 3, 1, 2), w.flip(2, 3) if flip else w, None if flip else bias, padding=1)
    ref = ref.permute(0, 2, 3, 1).reshape(B * H * W, N)
    assert int(err.item()) == 0
    assert _rel(y.cpu().numpy(), ref.numpy()) < 1e-5


def test_unet_implicit_and_explicit_paths_agree():
    from pylops_gb300.learned.unet import UNet

    g = torch.Generator().manual_seed(9)
    x = torch.randn(2, 64, 32, generator=g).cuda()
    t = torch.randn(2, 64, 32, generator=g).cuda()
    a, b = UNet(levels=4, base=16, seed=2, implicit=True), UNet(levels=4, base=16, seed=2, implicit=False)
    ya, yb = a.forward(x), b.forward(x)
    assert _rel(ya.cpu().numpy(), yb.cpu().numpy()) < 1e-2
    la, lb = float(a.loss_and_grad(x, t)), float(b.loss_and_grad(x, t))
    assert abs(la - lb) / lb < 1e-2
    for (wa, ba), (wb, bb) in zip(a.gradients(), b.gradients()):
        assert _rel(wa, wb) < 3e-2 and _rel(ba, bb) < 3e-2
    a.check_errors()
    b.check_errors()


@pytest.mark.parametrize("B,H,W,C,N", [(2, 8, 64, 32, 32), (1, 4, 128, 96, 64), (2, 6, 64, 64, 136),
                                       (1, 3, 64, 256, 16)])
def test_implicit_weight_gradient_matches_conv2d_weight(B, H, W, C, N):
    """kgb_unet_row_transpose + kgb_conv3x3_wgrad_bf16 (operands transposed
    per image row, x in three column-shifted copies stacked per row; rows
    (ky, kx, channel), split over pixels) against the weight gradient of torch conv2d (padding
    1) on the same bf16-rounded operands:
    dW[n][(ky*3 + kx)*C + c] = sum over pixels of g[p][n] x[p + (ky-1, kx-1)][c]."""
    from pylops_gb300 import _native

    g = torch.Generator().manual_seed(B * 100 + C + N)
    x = _bf(torch.randn(B, H, W, C, generator=g))
    gy = _bf(torch.randn(B, H, W, N, generator=g))
    ref = torch.nn.grad.conv2d_weight(x.permute(0, 3, 1, 2).double(), (N, C, 3, 3),
                                      gy.permute(0, 3, 1, 2).double(), padding=1)
    ref = ref.permute(0, 2, 3, 1).reshape(N, 9 * C).float()  # [n][(ky*3+kx)*C + c]
    P = B * H * W
    xd = x.to(torch.bfloat16).cuda().contiguous()
    gd = gy.to(torch.bfloat16).cuda().contiguous()
    xT3 = torch.empty(3 * P * C, dtype=torch.bfloat16, device="cuda")
    gTr = torch.empty(P * N, dtype=torch.bfloat16, device="cuda")
    ldw = 9 * C + 8
    dW = torch.full((N, ldw), 5.0, device="cuda")
    work = torch.empty(1 << 22, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    L, s = _native.lib(), torch.cuda.current_stream().cuda_stream
    _native.check(L.kgb_unet_row_transpose(xd.data_ptr(), xT3.data_ptr(), B, H, W, C, 3, s))
    _native.check(L.kgb_unet_row_transpose(gd.data_ptr(), gTr.data_ptr(), B, H, W, N, 1, s))
    # the transposed operands themselves: [b][h][shift][c][w] and [b][h][n][w]
    x3 = xT3.view(B, H, 3, C, W).float().cpu()
    xp = torch.nn.functional.pad(x.permute(0, 1, 3, 2), (1, 1))  # (B, H, C, W + 2)
    for kx in range(3):
        assert torch.equal(x3[:, :, kx], xp[..., kx:kx + W])
    assert torch.equal(gTr.view(B, H, N, W).float().cpu(), gy.permute(0, 1, 3, 2))
    _native.check(L.kgb_conv3x3_wgrad_bf16(xT3.data_ptr(), gTr.data_ptr(), dW.data_ptr(), B, H, W, C, N, ldw,
                                           work.data_ptr(), work.numel(), err.data_ptr(), s))
    got = dW.cpu()
    assert int(err.item()) == 0
    assert _rel(got[:, :9 * C].numpy(), ref.numpy()) < 1e-5
    assert torch.all(got[:, 9 * C:] == 5.0)


@pytest.mark.parametrize("B,Hg,Wg,C,N", [(2, 4, 128, 64, 32), (1, 3, 256, 32, 64), (2, 2, 128, 128, 64),
                                       (2, 2, 128, 64, 96), (2, 4, 64, 64, 32), (1, 8, 32, 128, 64),
                                       (3, 2, 64, 96, 64), (1, 4, 32, 40, 16)])
def test_stride2_data_gradient_matches_conv2d_input(B, Hg, Wg, C, N):
    """kgb_conv3x3_s2_dgrad_bf16 (four pixel-parity classes of implicit
    stride-1 convolutions on g) against the input gradient of torch conv2d
    (stride 2, padding 1) on the same bf16-rounded operands."""
    from pylops_gb300 import _native

    g = torch.Generator().manual_seed(B * 10 + C + N)
    w = _bf(torch.randn(C, N, 3, 3, generator=g) / (3 * N ** 0.5))  # forward weights: C outputs, N inputs
    gy = _bf(torch.randn(B, Hg, Wg, C, generator=g))
    ref = torch.nn.grad.conv2d_input((B, N, 2 * Hg, 2 * Wg), w.double(), gy.permute(0, 3, 1, 2).double(), stride=2,
                                     padding=1).permute(0, 2, 3, 1).float()
    Cp = (C + 63) // 64 * 64
    wt = torch.zeros(N, 9, Cp)
    wt[:, :, :C] = w.permute(1, 2, 3, 0).reshape(N, 9, C)  # Wti[n][tap * Cp + c] = W[c][n][tap]
    gd = gy.to(torch.bfloat16).cuda().contiguous()
    wd = wt.reshape(N, 9 * Cp).to(torch.bfloat16).cuda().contiguous()
    dx = torch.full((B, 2 * Hg, 2 * Wg, N), 3.0, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    _native.check(_native.lib().kgb_conv3x3_s2_dgrad_bf16(gd.data_ptr(), wd.data_ptr(), dx.data_ptr(), B, Hg, Wg, C,
                                                          N, err.data_ptr(),
                                                          torch.cuda.current_stream().cuda_stream))
    assert int(err.item()) == 0
    assert _rel(dx.cpu().numpy(), ref.numpy()) < 1e-5


def test_stride2_data_gradient_rejects_weights_that_do_not_fit():
    """Two 64-channel blocks of gradient channels with 128 output columns
    (288 KB of resident weights) are refused, and the network's layer check
    agrees (it keeps the unfolded GEMM for such layers)."""
    from pylops_gb300 import _native
    from pylops_gb300.learned.unet import _halo_weights_fit

    assert not _halo_weights_fit(128, 96) and _halo_weights_fit(128, 64) and _halo_weights_fit(64, 96)
    g = torch.zeros(1, 2, 128, 128, dtype=torch.bfloat16, device="cuda")
    wt = torch.zeros(96, 9 * 128, dtype=torch.bfloat16, device="cuda")
    dx = torch.zeros(1, 4, 256, 96, device="cuda")
    with pytest.raises(NotImplementedError):
        _native.check(_native.lib().kgb_conv3x3_s2_dgrad_bf16(g.data_ptr(), wt.data_ptr(), dx.data_ptr(), 1, 2, 128,
                                                              128, 96, None, torch.cuda.current_stream().cuda_stream))
    # 64-pixel rows need an even number of them (whole 128-pixel tiles per image)
    from pylops_gb300.learned.unet import _s2_tiles

    assert not _s2_tiles(3, 64) and _s2_tiles(4, 64) and _s2_tiles(8, 32) and not _s2_tiles(4, 96)
    with pytest.raises(ValueError):
        _native.check(_native.lib().kgb_conv3x3_s2_dgrad_bf16(g.data_ptr(), wt.data_ptr(), dx.data_ptr(), 1, 3, 64,
                                                              64, 32, None, torch.cuda.current_stream().cuda_stream))


@pytest.mark.parametrize("B,H,W,N", [(2, 16, 32, 32), (1, 9, 40, 8), (2, 8, 64, 16), (1, 8, 16, 64), (1, 5, 24, 24),
                                     (1, 4, 32, 128)])
def test_first_layer_kernels_match_conv2d(B, H, W, N):
    """kgb_unet_conv3x3_c1 (one input channel, N outputs, bias, ReLU, bf16
    NHWC output) and kgb_unet_conv3x3_c1_wgrad (pixel-parallel reduction for
    N = 8, 16, 32, 64; row-walking warps otherwise) against torch conv2d and
    its weight gradient in float64 on the same bf16-rounded operands."""
    from pylops_gb300 import _native

    gen = torch.Generator().manual_seed(B * 1000 + H * 10 + N)
    kpad = 16
    x = _bf(torch.randn(B, H, W, generator=gen))
    w = _bf(torch.randn(N, 9, generator=gen) / 3)
    bias = torch.randn(N, generator=gen) / 4
    gy = _bf(torch.randn(B, H, W, N, generator=gen))
    L, s = _native.lib(), torch.cuda.current_stream().cuda_stream
    xd = x.to(torch.bfloat16).cuda().contiguous()
    wd = torch.zeros(N, kpad, dtype=torch.bfloat16)
    wd[:, :9] = w.to(torch.bfloat16)
    wd = wd.cuda()
    bd = bias.cuda()
    # forward: relu(b + sum_t w[n][t] x[p + off(t)]) rounded to bf16
    y = torch.empty(B, H, W, N, dtype=torch.bfloat16, device="cuda")
    _native.check(L.kgb_unet_conv3x3_c1(xd.data_ptr(), wd.data_ptr(), bd.data_ptr(), y.data_ptr(), B, H, W, N, kpad, 1,
                                        s))
    ref = torch.nn.functional.conv2d(x[:, None].double(), w.view(N, 1, 3, 3).double(), bias.double(), padding=1)
    ref = torch.relu(ref).permute(0, 2, 3, 1).float()
    got = y.float().cpu()
    # float32 sums in tap order against float64, then bf16 rounding: at most one bf16 step apart
    assert torch.all((got - ref).abs() <= ref.abs() * 2.0 ** -7 + 1e-6)
    # weight gradient: dW[n][t] = sum over pixels of g[p][n] x[p + off(t)]; columns past 9 untouched
    gd = gy.to(torch.bfloat16).cuda().contiguous()
    dW = torch.full((N, kpad), 5.0, device="cuda")
    work = torch.empty(1 << 21, device="cuda")
    _native.check(L.kgb_unet_conv3x3_c1_wgrad(xd.data_ptr(), gd.data_ptr(), dW.data_ptr(), B, H, W, N, kpad,
                                              work.data_ptr(), s))
    refw = torch.nn.grad.conv2d_weight(x[:, None].double(), (N, 1, 3, 3), gy.permute(0, 3, 1, 2).double(), padding=1)
    gotw = dW.cpu()
    assert _rel(gotw[:, :9].numpy(), refw.view(N, 9).numpy()) < 1e-5
    assert torch.all(gotw[:, 9:] == 5.0)
    # deterministic: the same bits on a second call
    dW2 = torch.full((N, kpad), 5.0, device="cuda")
    _native.check(L.kgb_unet_conv3x3_c1_wgrad(xd.data_ptr(), gd.data_ptr(), dW2.data_ptr(), B, H, W, N, kpad,
                                              work.data_ptr(), s))
    assert torch.equal(dW2.cpu(), gotw)
