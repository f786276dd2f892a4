"""Learned warm start for SIRT-TV: a BF16 3D U-Net on hand-written tcgen05 kernels.

The network maps an FDK volume to a better starting image for SIRT-TV
(residual form: out = FDK + net(FDK)).  It is the one learned component of the
package and has no counterpart in the reference; plain SIRT-TV from the FDK
start stays the fallback, and the SIRT-TV data residual judges the network.

Architecture (4 levels, 32 base channels, 3x3x3 convolutions, ReLU):

    enc1: 1 -> 32 -> 32      (the 1-channel input enters as 27 gathered taps,
                              a 1-tap convolution over 32 channels)
    enc2: 32 -> 64 -> 64     after 2x max pooling
    enc3: 64 -> 128 -> 128
    bott: 128 -> 256 -> 256
    up:   1x1 convolution halving the channels, then nearest 2x upsampling
    dec3: [enc3, up] 256 -> 128 -> 128
    dec2: [enc2, up] 128 -> 64 -> 64
    dec1: [enc1, up] 64 -> 32 -> 32
    head: 1x1, 32 -> 1, added to the input

Every convolution, forward and both gradients, runs in ``ct_unet_conv3d`` /
``ct_unet_conv3d_wgrad`` (bf16 operands, FP32 accumulation in tensor memory);
pooling, upsampling, the head and the bias gradients are small CUDA kernels of
the same library.  PyTorch holds the tensors and runs Adam on the FP32 master
weights.  Activations are bf16 channels-last [n][z][y][x][c].
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import torch

from . import _lib
from .device import _stream

BF16 = torch.bfloat16


def _tptr(t: torch.Tensor):
    """Device pointer of a contiguous CUDA bf16 / float32 tensor."""
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if t.dtype not in (BF16, torch.float32):
        raise ValueError(f"expected a bfloat16 or float32 tensor, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return C.c_void_p(t.data_ptr())


def _p(t):
    return None if t is None else _tptr(t)


def status() -> int:
    """0 when no bounded wait of the convolutions gave up since the last call;
    otherwise raises CTError (CT_ERR_TIMEOUT).  Clears the device flag."""
    flags = C.c_int(0)
    _lib.call("ct_unet_status", C.byref(flags))
    return flags.value


def wait_selftest(limit_ns: int = 1_000_000) -> None:
    """Queue a bounded mbarrier wait on a barrier nothing arrives on (it gives up
    after ``limit_ns``); status() then raises CT_ERR_TIMEOUT with flag 8."""
    _lib.call("ct_unet_wait_selftest", int(limit_ns), C.c_void_p(torch.cuda.current_stream().cuda_stream))


# -- thin op wrappers ---------------------------------------------------------
def conv3d(x1, w, bias=None, relu=False, x2=None, ntaps=27, split=None, masks=(None, None)):
    """Convolution of concat(x1, x2) (bf16 [n][z][y][x][c]) with w (bf16
    [cout][taps][cin]); returns one output, or two when ``split`` = co1."""
    n, z, y, x, c1 = x1.shape
    c2 = 0 if x2 is None else x2.shape[-1]
    cout = w.shape[0]
    co1 = cout if split is None else split
    co2 = cout - co1
    out1 = torch.empty((n, z, y, x, co1), dtype=BF16, device=x1.device)
    out2 = torch.empty((n, z, y, x, co2), dtype=BF16, device=x1.device) if co2 else None
    _lib.call("ct_unet_conv3d", _tptr(x1), c1, _p(x2), c2, n, z, y, x, _tptr(w), ntaps, _p(bias), int(relu),
              _tptr(out1), co1, _p(out2), co2, _p(masks[0]), _p(masks[1]), _stream())
    return out1 if co2 == 0 else (out1, out2)


def shift_copies(xs, ntaps=27):
    """Channel-major x-shifted copies (xm, x0, xp) of the channel concat of xs."""
    n, z, y, x, _ = xs[0].shape
    ctot = sum(t.shape[-1] for t in xs)
    shape = (n, ctot, z, y, x)
    dev = xs[0].device
    x0 = torch.empty(shape, dtype=BF16, device=dev)
    xm = torch.empty(shape, dtype=BF16, device=dev) if ntaps == 27 else None
    xp = torch.empty(shape, dtype=BF16, device=dev) if ntaps == 27 else None
    off = 0
    for t in xs:
        c = t.shape[-1]
        _lib.call("ct_unet_shift_t", _tptr(t), c, n, z, y, x, _p(xm), _tptr(x0), _p(xp), ctot, off, _stream())
        off += c
    return xm, x0, xp


def conv3d_wgrad(xs, dy, ntaps=27, kper=None):
    """FP32 weight gradient [cout][taps][cin] of conv3d(concat(xs)) for output gradient dy."""
    n, z, y, x, cout = dy.shape
    xm, x0, xp = shift_copies(xs, ntaps)
    _, dyt, _ = shift_copies([dy], 1)
    cin = x0.shape[1]
    dw = torch.zeros((cout, ntaps, cin), dtype=torch.float32, device=dy.device)
    if kper is None:
        chunks = n * z * y * x // 64
        kper = max(16, -(-chunks // 1024))
    _lib.call("ct_unet_conv3d_wgrad", _p(xm), _tptr(x0), _p(xp), cin, _tptr(dyt), cout, n, z, y, x, ntaps, int(kper),
              _tptr(dw), _stream())
    return dw


def im2col27(vol):
    """fp32 [n][z][y][x] -> bf16 [n][z][y][x][32] of the 27 neighbours."""
    n, z, y, x = vol.shape
    out = torch.empty((n, z, y, x, 32), dtype=BF16, device=vol.device)
    _lib.call("ct_unet_im2col27", _tptr(vol), n, z, y, x, _tptr(out), _stream())
    return out


def pool2(t):
    n, z, y, x, c = t.shape
    out = torch.empty((n, z // 2, y // 2, x // 2, c), dtype=BF16, device=t.device)
    _lib.call("ct_unet_pool2", _tptr(t), _tptr(out), c, n, z // 2, y // 2, x // 2, _stream())
    return out


def pool2_bwd(x, y, dy):
    n, z, yy, xx, c = y.shape
    dx = torch.empty_like(x)
    _lib.call("ct_unet_pool2_bwd", _tptr(x), _tptr(y), _tptr(dy), _tptr(dx), c, n, z, yy, xx, _stream())
    return dx


def up2(t):
    n, z, y, x, c = t.shape
    out = torch.empty((n, 2 * z, 2 * y, 2 * x, c), dtype=BF16, device=t.device)
    _lib.call("ct_unet_up2", _tptr(t), _tptr(out), c, n, z, y, x, _stream())
    return out


def up2_bwd(dout):
    n, z, y, x, c = dout.shape
    din = torch.empty((n, z // 2, y // 2, x // 2, c), dtype=BF16, device=dout.device)
    _lib.call("ct_unet_up2_bwd", _tptr(dout), _tptr(din), c, n, z // 2, y // 2, x // 2, _stream())
    return din


def head(f, w, b, base):
    out = torch.empty(f.shape[:-1], dtype=torch.float32, device=f.device)
    _lib.call("ct_unet_head", _tptr(f), _tptr(w), _tptr(b), _p(base), _tptr(out), out.numel(), _stream())
    return out


def head_bwd(dout, f, w, dw, db):
    df = torch.empty_like(f)
    _lib.call("ct_unet_head_bwd", _tptr(dout), _tptr(f), _tptr(w), _tptr(df), _tptr(dw), _tptr(db), dout.numel(),
              _stream())
    return df


def colsum(dy, db):
    c = dy.shape[-1]
    _lib.call("ct_unet_colsum", _tptr(dy), c, dy.numel() // c, _tptr(db), _stream())


# -- the network ----------------------------------------------------------------
# (name, cin, cout, taps, relu)
LAYERS = [
    ("e1a", 32, 32, 1, True), ("e1b", 32, 32, 27, True),
    ("e2a", 32, 64, 27, True), ("e2b", 64, 64, 27, True),
    ("e3a", 64, 128, 27, True), ("e3b", 128, 128, 27, True),
    ("b1", 128, 256, 27, True), ("b2", 256, 256, 27, True),
    ("u3", 256, 128, 1, False), ("d3a", 256, 128, 27, True), ("d3b", 128, 128, 27, True),
    ("u2", 128, 64, 1, False), ("d2a", 128, 64, 27, True), ("d2b", 64, 64, 27, True),
    ("u1", 64, 32, 1, False), ("d1a", 64, 32, 27, True), ("d1b", 32, 32, 27, True),
]


_RELU = {name: relu for name, _, _, _, relu in LAYERS}


def flops_per_voxel() -> float:
    """Multiply-adds x 2 of one forward pass per full-resolution voxel."""
    level = {"e1": 1, "d1": 1, "u1": 8, "e2": 8, "d2": 8, "u2": 64, "e3": 64, "d3": 64, "u3": 512, "b": 512}
    total = 0.0
    for name, cin, cout, taps, _ in LAYERS:
        key = next(k for k in level if name.startswith(k))
        total += 2.0 * cin * cout * taps / level[key]
    return total + 2.0 * 32


@dataclass
class AdamState:
    lr: float = 1e-3
    b1: float = 0.9
    b2: float = 0.999
    eps: float = 1e-8
    t: int = 0
    m: dict = field(default_factory=dict)
    v: dict = field(default_factory=dict)


class UNet3D:
    """The warm-start network: FP32 master weights, bf16 copies for the kernels."""

    def __init__(self, seed: int = 0, device="cuda"):
        g = torch.Generator().manual_seed(seed)
        self.device = torch.device(device)
        self.params: dict[str, torch.Tensor] = {}
        for name, cin, cout, taps, _ in LAYERS:
            fan_in = (27 if name == "e1a" else taps * cin)
            w = torch.randn((cout, taps, cin), generator=g) * math.sqrt(2.0 / fan_in)
            if name == "e1a":
                w[:, :, 27:] = 0.0           # the 5 padding channels of the gathered input
            self.params[name + ".w"] = w.to(self.device)
            self.params[name + ".b"] = torch.zeros(cout, device=self.device)
        # zero head: the untrained network returns its input
        self.params["head.w"] = torch.zeros(32, device=self.device)
        self.params["head.b"] = torch.zeros(1, device=self.device)
        self.adam = AdamState()
        self._refresh()

    def _refresh(self):
        self.wb = {k[:-2]: v.to(BF16).contiguous() for k, v in self.params.items() if k.endswith(".w")
                   and not k.startswith("head")}
        self.wt = {}   # flipped / transposed weights of the data gradient, built lazily

    def _wt(self, name):
        if name not in self.wt:
            w = self.wb[name]                            # [cout][taps][cin]
            self.wt[name] = w.flip(1).transpose(0, 2).contiguous()   # [cin][taps][cout], taps reversed
        return self.wt[name]

    def state_dict(self):
        return {k: v.detach().cpu() for k, v in self.params.items()}

    def load_state_dict(self, sd):
        for k in self.params:
            self.params[k] = sd[k].to(self.device).float()
        self._refresh()

    # forward -------------------------------------------------------------------
    def _conv(self, name, *xs, ntaps):
        return conv3d(xs[0], self.wb[name], self.params[name + ".b"], relu=_RELU[name],
                      x2=xs[1] if len(xs) > 1 else None, ntaps=ntaps)

    def forward(self, x: torch.Tensor, keep: bool = False):
        """x: fp32 [n][z][y][x] or [z][y][x] (sizes multiples of 16) -> fp32 [n][z][y][x].
        keep=True saves the activations for backward()."""
        if x.dim() == 3:
            x = x.unsqueeze(0)
        if x.dim() != 4 or any(d % 16 for d in x.shape[1:]):
            raise ValueError(f"U-Net input must be [n][z][y][x] with sizes multiples of 16 (three 2x poolings, "
                             f"8-voxel tiles at the coarsest level); got {tuple(x.shape)}")
        x = x.contiguous()
        a = {"x": x}
        a["g"] = im2col27(x)
        a["e1a"] = self._conv("e1a", a["g"], ntaps=1)
        a["e1"] = self._conv("e1b", a["e1a"], ntaps=27)
        a["p1"] = pool2(a["e1"])
        a["e2a"] = self._conv("e2a", a["p1"], ntaps=27)
        a["e2"] = self._conv("e2b", a["e2a"], ntaps=27)
        a["p2"] = pool2(a["e2"])
        a["e3a"] = self._conv("e3a", a["p2"], ntaps=27)
        a["e3"] = self._conv("e3b", a["e3a"], ntaps=27)
        a["p3"] = pool2(a["e3"])
        a["b1"] = self._conv("b1", a["p3"], ntaps=27)
        a["b2"] = self._conv("b2", a["b1"], ntaps=27)
        a["c3"] = self._conv("u3", a["b2"], ntaps=1)
        a["up3"] = up2(a["c3"])
        a["d3a"] = self._conv("d3a", a["e3"], a["up3"], ntaps=27)
        a["d3"] = self._conv("d3b", a["d3a"], ntaps=27)
        a["c2"] = self._conv("u2", a["d3"], ntaps=1)
        a["up2"] = up2(a["c2"])
        a["d2a"] = self._conv("d2a", a["e2"], a["up2"], ntaps=27)
        a["d2"] = self._conv("d2b", a["d2a"], ntaps=27)
        a["c1"] = self._conv("u1", a["d2"], ntaps=1)
        a["up1"] = up2(a["c1"])
        a["d1a"] = self._conv("d1a", a["e1"], a["up1"], ntaps=27)
        a["d1"] = self._conv("d1b", a["d1a"], ntaps=27)
        out = head(a["d1"], self.params["head.w"], self.params["head.b"], x)
        self.cache = a if keep else None
        return out

    __call__ = forward

    # backward ------------------------------------------------------------------
    def backward(self, dout: torch.Tensor) -> dict:
        """Gradients of all parameters for d(loss)/d(out) = dout (fp32, the output's shape)."""
        a = self.cache
        if a is None:
            raise RuntimeError("backward needs forward(..., keep=True)")
        grads = {k: torch.zeros_like(v) for k, v in self.params.items()}

        def wgrad(name, xs, dy, ntaps):
            grads[name + ".w"] += conv3d_wgrad(xs, dy, ntaps)
            colsum(dy, grads[name + ".b"])

        dout = dout.reshape(a["x"].shape).contiguous()
        dd1 = head_bwd(dout, a["d1"], self.params["head.w"], grads["head.w"], grads["head.b"])   # masked by d1 > 0
        # dec1
        wgrad("d1b", [a["d1a"]], dd1, 27)
        dd1a = conv3d(dd1, self._wt("d1b"), masks=(a["d1a"], None))
        wgrad("d1a", [a["e1"], a["up1"]], dd1a, 27)
        de1_skip, dup1 = conv3d(dd1a, self._wt("d1a"), split=32, masks=(a["e1"], None))
        dc1 = up2_bwd(dup1)
        wgrad("u1", [a["d2"]], dc1, 1)
        dd2 = conv3d(dc1, self._wt("u1"), ntaps=1, masks=(a["d2"], None))
        # dec2
        wgrad("d2b", [a["d2a"]], dd2, 27)
        dd2a = conv3d(dd2, self._wt("d2b"), masks=(a["d2a"], None))
        wgrad("d2a", [a["e2"], a["up2"]], dd2a, 27)
        de2_skip, dup2 = conv3d(dd2a, self._wt("d2a"), split=64, masks=(a["e2"], None))
        dc2 = up2_bwd(dup2)
        wgrad("u2", [a["d3"]], dc2, 1)
        dd3 = conv3d(dc2, self._wt("u2"), ntaps=1, masks=(a["d3"], None))
        # dec3
        wgrad("d3b", [a["d3a"]], dd3, 27)
        dd3a = conv3d(dd3, self._wt("d3b"), masks=(a["d3a"], None))
        wgrad("d3a", [a["e3"], a["up3"]], dd3a, 27)
        de3_skip, dup3 = conv3d(dd3a, self._wt("d3a"), split=128, masks=(a["e3"], None))
        dc3 = up2_bwd(dup3)
        wgrad("u3", [a["b2"]], dc3, 1)
        db2 = conv3d(dc3, self._wt("u3"), ntaps=1, masks=(a["b2"], None))
        # bottleneck
        wgrad("b2", [a["b1"]], db2, 27)
        db1 = conv3d(db2, self._wt("b2"), masks=(a["b1"], None))
        wgrad("b1", [a["p3"]], db1, 27)
        dp3 = conv3d(db1, self._wt("b1"))
        # enc3: the skip path is masked by e3 > 0 in its epilogue; the pooling
        # gradient reaches only window maxima that are > 0
        de3 = de3_skip + pool2_bwd(a["e3"], a["p3"], dp3)
        wgrad("e3b", [a["e3a"]], de3, 27)
        de3a = conv3d(de3, self._wt("e3b"), masks=(a["e3a"], None))
        wgrad("e3a", [a["p2"]], de3a, 27)
        dp2 = conv3d(de3a, self._wt("e3a"))
        de2 = de2_skip + pool2_bwd(a["e2"], a["p2"], dp2)
        wgrad("e2b", [a["e2a"]], de2, 27)
        de2a = conv3d(de2, self._wt("e2b"), masks=(a["e2a"], None))
        wgrad("e2a", [a["p1"]], de2a, 27)
        dp1 = conv3d(de2a, self._wt("e2a"))
        de1 = de1_skip + pool2_bwd(a["e1"], a["p1"], dp1)
        wgrad("e1b", [a["e1a"]], de1, 27)
        de1a = conv3d(de1, self._wt("e1b"), masks=(a["e1a"], None))
        wgrad("e1a", [a["g"]], de1a, 1)
        grads["e1a.w"][:, :, 27:] = 0.0
        return grads

    def adam_step(self, grads: dict, lr: float | None = None):
        s = self.adam
        s.t += 1
        lr = s.lr if lr is None else lr
        c1 = 1.0 - s.b1 ** s.t
        c2 = 1.0 - s.b2 ** s.t
        for k, p in self.params.items():
            g = grads[k]
            m = s.m.setdefault(k, torch.zeros_like(p))
            v = s.v.setdefault(k, torch.zeros_like(p))
            m.mul_(s.b1).add_(g, alpha=1 - s.b1)
            v.mul_(s.b2).addcmul_(g, g, value=1 - s.b2)
            p.addcdiv_(m / c1, (v / c2).sqrt_().add_(s.eps), value=-lr)
        self._refresh()


# -- FP32 reference of the same network (tests) ---------------------------------
def reference_forward(params: dict, x: torch.Tensor, round_bf16: bool = True) -> torch.Tensor:
    """torch.nn.functional restatement of UNet3D.forward in FP32 (NCDHW), with
    activations and weights rounded to bf16 where the kernels store bf16."""
    import torch.nn.functional as F

    def r(t):
        return t.to(BF16).float() if round_bf16 else t

    def conv(name, t, taps, relu):
        w = r(params[name + ".w"])                              # [cout][taps][cin]
        cout, _, cin = w.shape
        k = 3 if taps == 27 else 1
        wt = w.permute(0, 2, 1).reshape(cout, cin, k, k, k)
        y = F.conv3d(t, wt, params[name + ".b"], padding=k // 2)
        return r(F.relu(y) if relu else y)

    if x.dim() == 3:
        x = x.unsqueeze(0)
    xin = x.unsqueeze(1).float()
    taps = []
    xp = F.pad(xin, (1, 1, 1, 1, 1, 1))
    Z, Y, X = x.shape[1:]
    for k in range(27):
        dz, dy, dx = k // 9, (k // 3) % 3, k % 3
        taps.append(xp[:, :, dz:dz + Z, dy:dy + Y, dx:dx + X])
    g = r(torch.cat(taps + [torch.zeros_like(xin)] * 5, 1))
    e1 = conv("e1b", conv("e1a", g, 1, True), 27, True)
    e2 = conv("e2b", conv("e2a", F.max_pool3d(e1, 2), 27, True), 27, True)
    e3 = conv("e3b", conv("e3a", F.max_pool3d(e2, 2), 27, True), 27, True)
    b2 = conv("b2", conv("b1", F.max_pool3d(e3, 2), 27, True), 27, True)
    up = F.interpolate(conv("u3", b2, 1, False), scale_factor=2, mode="nearest")
    d3 = conv("d3b", conv("d3a", torch.cat([e3, up], 1), 27, True), 27, True)
    up = F.interpolate(conv("u2", d3, 1, False), scale_factor=2, mode="nearest")
    d2 = conv("d2b", conv("d2a", torch.cat([e2, up], 1), 27, True), 27, True)
    up = F.interpolate(conv("u1", d2, 1, False), scale_factor=2, mode="nearest")
    d1 = conv("d1b", conv("d1a", torch.cat([e1, up], 1), 27, True), 27, True)
    out = (d1 * params["head.w"].view(1, 32, 1, 1, 1)).sum(1) + params["head.b"] + x.float()
    return out
