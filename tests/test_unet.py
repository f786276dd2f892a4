"""The warm-start U-Net's kernels (ctgb/unet.py, csrc/unet_conv.cu, csrc/unet_ops.cu).

The tensor-core convolution is checked against torch's FP32 conv3d on the same
bf16 values: products of bf16 numbers are exact in FP32, so the kernel and the
reference differ only in FP32 summation order, and after rounding to bf16
almost every output is bit-identical (rel-L2 <= 2e-3 and >= 99% equal).  The
FP32 weight gradient is compared at rel-L2 <= 1e-4.  The whole network is
compared with a torch restatement that rounds activations to bf16 where the
kernels store them (rel-L2 <= 1e-2 forward, <= 5e-2 per gradient).
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2

BF = torch.bfloat16


def _t2ndhwc(t):        # torch NCDHW -> channels-last
    return t.permute(0, 2, 3, 4, 1).contiguous()


def _ndhwc2t(t):
    return t.permute(0, 4, 1, 2, 3).contiguous()


def _w2torch(w):        # [cout][taps][cin] -> [cout][cin][k][k][k]
    cout, taps, cin = w.shape
    k = 3 if taps == 27 else 1
    return w.permute(0, 2, 1).reshape(cout, cin, k, k, k)


def test_flops_and_layer_table():
    from ctgb import unet
    names = [n for n, *_ in unet.LAYERS]
    assert len(names) == len(set(names)) == 17
    # every 3x3x3 layer's input channels are what the previous stage produces
    assert dict((n, (ci, co)) for n, ci, co, *_ in unet.LAYERS)["d1a"] == (64, 32)
    f = unet.flops_per_voxel()
    assert 4.0e5 < f < 8.0e5


def test_reference_network_starts_as_identity():
    from ctgb import unet
    net_params = {}
    g = torch.Generator().manual_seed(0)
    for name, cin, cout, taps, _ in unet.LAYERS:
        net_params[name + ".w"] = torch.randn((cout, taps, cin), generator=g) * 0.05
        net_params[name + ".b"] = torch.zeros(cout)
    net_params["head.w"] = torch.zeros(32)
    net_params["head.b"] = torch.zeros(1)
    x = torch.rand((1, 16, 16, 16))
    out = unet.reference_forward(net_params, x)
    assert torch.equal(out, x)


FWD_CASES = [
    # c1, c2, cout, taps, nb, nz, ny, nx, split, masked
    (32, 0, 32, 27, 1, 4, 8, 16, None, False),
    (64, 64, 128, 27, 2, 3, 8, 32, 64, True),
    (256, 0, 256, 27, 1, 2, 16, 8, None, False),
    (32, 0, 64, 1, 1, 2, 4, 128, None, False),
    (128, 0, 32, 27, 1, 2, 2, 256, None, True),
    (32, 32, 64, 27, 1, 5, 16, 16, 32, True),
    (64, 0, 128, 27, 1, 8, 4, 8, None, False),       # 128-voxel tiles spanning 4 slices
    # y-halo tiles (x a multiple of 8, y of 16, <= 128 outputs): one box per (dz, dx) for 3 dy taps
    (64, 0, 128, 27, 2, 3, 32, 24, None, False),
    (32, 0, 32, 27, 1, 2, 48, 8, None, True),
    (128, 128, 128, 27, 1, 2, 16, 16, 96, True),
]


@pytest.mark.gpu
@pytest.mark.parametrize("c1,c2,cout,taps,nb,nz,ny,nx,split,masked", FWD_CASES)
def test_conv3d_matches_torch(c1, c2, cout, taps, nb, nz, ny, nx, split, masked):
    import torch.nn.functional as F
    from ctgb import unet
    g = torch.Generator(device="cuda").manual_seed(c1 + 7 * cout + nx)
    x1 = torch.randn((nb, nz, ny, nx, c1), device="cuda", generator=g).to(BF)
    x2 = torch.randn((nb, nz, ny, nx, c2), device="cuda", generator=g).to(BF) if c2 else None
    w = (torch.randn((cout, taps, c1 + c2), device="cuda", generator=g) / np.sqrt(taps * (c1 + c2))).to(BF)
    bias = torch.randn(cout, device="cuda", generator=g) * 0.1
    relu = not masked
    masks = (None, None)
    if masked:
        m = torch.randn((nb, nz, ny, nx, cout), device="cuda", generator=g).to(BF)
        masks = (m[..., :split].contiguous(), m[..., split:].contiguous()) if split else (m, None)
    out = unet.conv3d(x1, w, bias, relu=relu, x2=x2, ntaps=taps, split=split, masks=masks)
    torch.cuda.synchronize()
    assert unet.status() == 0
    out = torch.cat(out, -1) if split else out
    xt = _ndhwc2t(torch.cat([x1, x2], -1) if c2 else x1).float()
    ref = F.conv3d(xt, _w2torch(w.float()), bias, padding=1 if taps == 27 else 0)
    ref = _t2ndhwc(F.relu(ref) if relu else ref)
    if masked:
        mm = torch.cat(masks, -1) if split else masks[0]
        ref = torch.where(mm.float() > 0, ref, torch.zeros_like(ref))
    ref = ref.to(BF)
    assert rel_l2(out.float().cpu().numpy(), ref.float().cpu().numpy()) <= 2e-3
    assert (out == ref).float().mean().item() >= 0.99


WGRAD_CASES = [
    # cins (concat parts), cout, taps, nb, nz, ny, nx, kper
    ((32,), 32, 27, 1, 4, 8, 16, 3),
    ((64, 64), 128, 27, 2, 3, 8, 32, 5),
    ((256,), 256, 27, 1, 4, 8, 8, 2),
    ((32,), 64, 1, 1, 2, 16, 16, 4),
    ((128,), 32, 27, 1, 2, 2, 64, 1),
    ((32, 32), 64, 27, 1, 5, 16, 16, None),
    ((64,), 128, 27, 2, 3, 4, 8, 1),                # y*x = 32: one slice runs past each plane
    ((32,), 32, 27, 1, 2, 12, 8, 2),                # y*x = 96: the last slice is half outside
]


@pytest.mark.gpu
@pytest.mark.parametrize("cins,cout,taps,nb,nz,ny,nx,kper", WGRAD_CASES)
def test_conv3d_wgrad_matches_autograd(cins, cout, taps, nb, nz, ny, nx, kper):
    import torch.nn.functional as F
    from ctgb import unet
    g = torch.Generator(device="cuda").manual_seed(sum(cins) + cout + nx)
    xs = [torch.randn((nb, nz, ny, nx, c), device="cuda", generator=g).to(BF) for c in cins]
    dy = torch.randn((nb, nz, ny, nx, cout), device="cuda", generator=g).to(BF)
    dw = unet.conv3d_wgrad(xs, dy, taps, kper=kper)
    torch.cuda.synchronize()
    assert unet.status() == 0
    cin = sum(cins)
    wt = torch.zeros((cout, taps, cin), device="cuda", requires_grad=True)
    xt = _ndhwc2t(torch.cat(xs, -1)).float()
    y = F.conv3d(xt, _w2torch(wt), padding=1 if taps == 27 else 0)
    y.backward(_ndhwc2t(dy).float())
    assert rel_l2(dw.cpu().numpy(), wt.grad.cpu().numpy()) <= 1e-4


@pytest.mark.gpu
def test_shift_copies_past_65535_rows():
    """The channel-major x-shifted copies for more than 65535 (n, z, y) rows
    (a 256^3 training volume has 65536)."""
    from ctgb import unet
    g = torch.Generator(device="cuda").manual_seed(12)
    t = torch.randn((1, 64, 1040, 8, 32), device="cuda", generator=g).to(BF)
    xm, x0, xp = unet.shift_copies([t])
    ref = t.permute(0, 4, 1, 2, 3)                                   # [n][c][z][y][x]
    assert torch.equal(x0, ref)
    assert torch.equal(xm[..., 1:], ref[..., :-1]) and torch.count_nonzero(xm[..., 0]) == 0
    assert torch.equal(xp[..., :-1], ref[..., 1:]) and torch.count_nonzero(xp[..., -1]) == 0


@pytest.mark.gpu
def test_elementwise_ops_match_torch():
    import torch.nn.functional as F
    from ctgb import unet
    g = torch.Generator(device="cuda").manual_seed(5)
    vol = torch.rand((2, 6, 8, 16), device="cuda", generator=g)
    col = unet.im2col27(vol)
    xp = F.pad(vol, (1, 1, 1, 1, 1, 1))
    for k in (0, 4, 13, 22, 26):
        dz, dy, dx = k // 9, (k // 3) % 3, k % 3
        assert torch.equal(col[..., k], xp[:, dz:dz + 6, dy:dy + 8, dx:dx + 16].to(BF))
    assert torch.count_nonzero(col[..., 27:]) == 0
    # pooling of ReLU outputs (ties and zero windows included) and its gradient
    x = F.relu(torch.randn((1, 8, 8, 16, 16), device="cuda", generator=g)).round(decimals=1).to(BF)
    y = unet.pool2(x)
    xt = _ndhwc2t(x).float().requires_grad_(True)
    yt = F.max_pool3d(xt, 2)
    assert torch.equal(y.float(), _t2ndhwc(yt.detach()))
    dy = torch.randn(y.shape, device="cuda", generator=g).to(BF)
    dx = unet.pool2_bwd(x, y, dy)
    # each window passes its gradient to exactly one maximum, when that maximum is > 0
    win = dx.float().reshape(1, 4, 2, 4, 2, 8, 2, 16).permute(0, 1, 3, 5, 7, 2, 4, 6).reshape(1, 4, 4, 8, 16, 8)
    nz = (win != 0).sum(-1)
    assert int(nz.max()) <= 1
    got = win.sum(-1)
    want = torch.where(y.float() > 0, dy.float(), torch.zeros_like(dy.float()))
    assert torch.equal(got, want)
    pos = dx.float() != 0
    assert torch.equal(x.float()[pos], y.float().reshape(1, 4, 1, 4, 1, 8, 1, 16).expand(1, 4, 2, 4, 2, 8, 2, 16)
                       .reshape(x.shape)[pos])
    # nearest upsampling and its gradient
    u = unet.up2(y)
    assert torch.equal(_ndhwc2t(u).float(), F.interpolate(_ndhwc2t(y).float(), scale_factor=2, mode="nearest"))
    du = torch.randn(u.shape, device="cuda", generator=g).to(BF)
    dyu = unet.up2_bwd(du)
    ref = du.float().reshape(1, 4, 2, 4, 2, 8, 2, 16).sum((2, 4, 6)).to(BF)
    assert rel_l2(dyu.float().cpu().numpy(), ref.float().cpu().numpy()) <= 4e-3
    # head and its gradient
    f = F.relu(torch.randn((1, 4, 8, 16, 32), device="cuda", generator=g)).to(BF)
    w = torch.randn(32, device="cuda", generator=g)
    b = torch.randn(1, device="cuda", generator=g)
    base = torch.rand((1, 4, 8, 16), device="cuda", generator=g)
    out = unet.head(f, w, b, base)
    ref = (f.float() * w).sum(-1) + b + base
    assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) <= 1e-6
    dout = torch.randn(out.shape, device="cuda", generator=g)
    dw = torch.zeros(32, device="cuda")
    db = torch.zeros(1, device="cuda")
    df = unet.head_bwd(dout, f, w, dw, db)
    assert rel_l2(dw.cpu().numpy(), (dout[..., None] * f.float()).sum((0, 1, 2, 3)).cpu().numpy()) <= 1e-5
    assert float(db) == pytest.approx(float(dout.sum()), rel=1e-5)
    ref_df = torch.where(f.float() > 0, w * dout[..., None], torch.zeros_like(f.float())).to(BF)
    assert torch.equal(df, ref_df)
    # bias gradient
    for c in (32, 64, 128, 256):
        t = torch.randn((1, 3, 4, 8, c), device="cuda", generator=g).to(BF)
        s = torch.zeros(c, device="cuda")
        unet.colsum(t, s)
        assert rel_l2(s.cpu().numpy(), t.float().sum((0, 1, 2, 3)).cpu().numpy()) <= 1e-5


@pytest.mark.gpu
def test_network_forward_and_gradients_match_torch():
    from ctgb import unet
    net = unet.UNet3D(seed=3)
    g = torch.Generator(device="cuda").manual_seed(9)
    for k in net.params:                        # nonzero biases and head so every path carries gradient
        if k.endswith(".b") or k.startswith("head"):
            net.params[k] = 0.05 * torch.randn(net.params[k].shape, device="cuda", generator=g)
    net._refresh()
    x = torch.rand((1, 32, 32, 64), device="cuda", generator=g)
    out = net.forward(x, keep=True)
    torch.cuda.synchronize()
    assert unet.status() == 0
    params = {k: v.clone().requires_grad_(True) for k, v in net.params.items()}
    ref = unet.reference_forward(params, x)
    assert rel_l2(out.cpu().numpy(), ref.detach().cpu().numpy()) <= 1e-2
    target = torch.rand_like(x)
    dout = 2.0 * (out - target) / out.numel()
    grads = net.backward(dout)
    torch.cuda.synchronize()
    assert unet.status() == 0
    loss = ((ref - target) ** 2).mean()
    loss.backward()
    for k, p in params.items():
        ref_g = p.grad.cpu().numpy()
        if k == "e1a.w":
            ref_g[:, :, 27:] = 0.0
        assert rel_l2(grads[k].cpu().numpy(), ref_g) <= 5e-2, k


@pytest.mark.gpu
def test_training_steps_reduce_loss():
    """Adam on the hand-written gradients fits an affine map of the input."""
    from ctgb import phantom, unet
    net = unet.UNet3D(seed=1)
    x = phantom.ellipsoids_3d(64, 64, 64, phantom.ellipsoid_params(6, seed=4), device="cuda")[None]
    target = 0.8 * x + 0.05
    losses = []
    for _ in range(25):
        out = net.forward(x, keep=True)
        losses.append(float(((out - target) ** 2).mean()))
        net.adam_step(net.backward(2.0 * (out - target) / out.numel()), lr=3e-4)
    torch.cuda.synchronize()
    assert unet.status() == 0
    assert min(losses[-5:]) < 0.6 * losses[0], losses


def test_network_rejects_sizes_it_cannot_pool():
    from ctgb import unet
    net = unet.UNet3D(seed=0, device="cpu")
    with pytest.raises(ValueError, match="multiples of 16"):
        net.forward(torch.zeros((1, 24, 32, 32)))


@pytest.mark.gpu
def test_bounded_wait_gives_up_and_reports_timeout():
    """A bounded mbarrier wait on a barrier that nothing arrives on gives up after
    its limit (1 ms here), the host reads CT_ERR_TIMEOUT, the flag clears, and
    the context keeps working: a convolution afterwards is still correct."""
    import time
    import torch.nn.functional as F
    from ctgb import unet
    from ctgb._lib import CTError
    torch.cuda.synchronize()
    assert unet.status() == 0
    t0 = time.perf_counter()
    unet.wait_selftest(1_000_000)
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 5.0
    with pytest.raises(CTError) as e:
        unet.status()
    assert e.value.status == 5 and "flags 8" in str(e.value)
    assert unet.status() == 0                     # read-and-clear
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn((1, 2, 8, 16, 32), device="cuda", generator=g).to(BF)
    w = (torch.randn((32, 27, 32), device="cuda", generator=g) / np.sqrt(27 * 32)).to(BF)
    out = unet.conv3d(x, w, torch.zeros(32, device="cuda"), relu=False)
    torch.cuda.synchronize()
    assert unet.status() == 0
    ref = _t2ndhwc(F.conv3d(_ndhwc2t(x).float(), _w2torch(w.float()), None, padding=1)).to(BF)
    assert rel_l2(out.float().cpu().numpy(), ref.float().cpu().numpy()) <= 2e-3
