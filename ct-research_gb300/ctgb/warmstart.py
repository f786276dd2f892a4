"""Learned warm start for sparse-view cone-beam SIRT-TV.

The method generates its own training set: random-ellipsoid phantoms are
projected by the Siddon forward projector over a sparse (90-view) scan,
reconstructed by FDK (the network input) and by SIRT-TV (the target), both on
this package's operators.  The BF16 U-Net (``unet.UNet3D``) is trained on the
pairs, and at inference its output replaces the FDK volume as the starting
image of SIRT-TV.  Plain SIRT-TV from the FDK start is the fallback and the
yardstick: both starts run the same loop (``sirt.AsdLoop``) to the same
relative data residual, and the data residual alone decides when a run is done.

The training scan is the 512^3 workload's scan (200 x 200 x 150 mm, 768 x 512
detector at 0.8 mm, SID 600 / SDD 1200) with n^3 voxels and the detector
scaled by n / 512.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np
import torch
import torch.nn.functional as F

from . import phantom, unet
from .device import ConePlan
from .geometry import ConeGeometry, cone_from_physical
from .sirt import AsdConfig, AsdLoop

SIZE_MM = (200.0, 200.0, 150.0)
WEIGHTS = Path(__file__).resolve().parent / "weights" / "warmstart_unet.npz"


def scan(n: int, views: int = 90) -> ConeGeometry:
    """n^3 voxels over 200 x 200 x 150 mm; (768, 512) * n / 512 detector bins at
    0.8 * 512 / n mm; SID 600, SDD 1200; views over 360 degrees."""
    f = n / 512.0
    return cone_from_physical((n, n, n), SIZE_MM, views, int(round(768 * f)), int(round(512 * f)), 0.8 / f, 600.0,
                              1200.0, name=f"cone_{n}_{views}v")


def phantom_volume(n: int, seed: int, count: int = 12, device="cuda") -> torch.Tensor:
    return phantom.ellipsoids_3d(n, n, n, phantom.ellipsoid_params(count, seed=seed), device=device).contiguous()


@dataclass
class PairSet:
    inputs: torch.Tensor          # [N][n][n][n] fp32 FDK volumes
    targets: torch.Tensor         # [N][n][n][n] fp32 SIRT-TV volumes
    seeds: list = field(default_factory=list)
    residuals: list = field(default_factory=list)   # final relative data residual of each target
    seconds: float = 0.0


def generate(n_pairs: int, n: int = 128, views: int = 90, iters: int = 500, seed0: int = 1000,
             cfg: AsdConfig | None = None, log=None) -> PairSet:
    """n_pairs (FDK, SIRT-TV) pairs from phantoms of seeds seed0, seed0 + 1, ..."""
    plan = ConePlan(scan(n, views))
    loop = AsdLoop(plan, cfg or AsdConfig(iters=iters), use_graph=True)
    inputs = torch.empty((n_pairs, n, n, n), dtype=torch.float32, device="cuda")
    targets = torch.empty_like(inputs)
    out = PairSet(inputs, targets)
    t0 = time.perf_counter()
    for i in range(n_pairs):
        seed = seed0 + i
        vol = phantom_volume(n, seed)
        b = plan.fp(vol)
        x0 = plan.fdk(b)
        res = loop.run(b, x0, iters=iters, check_every=iters)
        inputs[i].copy_(x0)
        targets[i].copy_(res.x)
        out.seeds.append(seed)
        out.residuals.append(res.residuals[-1][1])
        if log and (i % 50 == 0 or i == n_pairs - 1):
            log(f"pair {i + 1}/{n_pairs}: residual after {iters} iterations {res.residuals[-1][1]:.3e}, "
                f"{time.perf_counter() - t0:.1f} s")
    torch.cuda.synchronize()
    out.seconds = time.perf_counter() - t0
    return out


def train(net: unet.UNet3D, pairs: PairSet, epochs: int = 4, lr: float = 3e-4, lr_end: float = 3e-5, seed: int = 0,
          log=None, on_epoch=None) -> list:
    """Adam on the mean squared error to the SIRT-TV targets, one pair per step,
    cosine learning-rate decay from lr to lr_end; returns the mean loss per epoch.

    Each step flips the pair along a random subset of the axes and may swap x
    and y.  A flip of x or y maps the view angles b to -b or pi - b, which keeps
    the 90-view set (multiples of 4 degrees), and a flip of z keeps the central
    orbit: the flipped pair is another (FDK, SIRT-TV) pair of the same scan.
    The x-y swap maps b to 3 pi / 2 - b, i.e. the same scan with its views
    turned by half a view step (2 degrees): still a 90-view pair of this
    geometry."""
    n_pairs = pairs.inputs.shape[0]
    total = epochs * n_pairs
    rng = np.random.default_rng(seed)
    history = []
    step = 0
    for ep in range(epochs):
        order = rng.permutation(n_pairs)
        acc = torch.zeros((), dtype=torch.float64, device="cuda")
        for i in order:
            x = pairs.inputs[i:i + 1]
            y = pairs.targets[i:i + 1]
            dims = [d for d in (1, 2, 3) if rng.random() < 0.5]
            if dims:
                x, y = x.flip(dims), y.flip(dims)
            if rng.random() < 0.5:
                x, y = x.transpose(2, 3), y.transpose(2, 3)
            x, y = x.contiguous(), y.contiguous()
            out = net.forward(x, keep=True)
            diff = out - y
            acc += (diff.double() ** 2).mean()
            cur = lr_end + 0.5 * (lr - lr_end) * (1.0 + math.cos(math.pi * step / max(1, total - 1)))
            net.adam_step(net.backward(2.0 * diff / diff.numel()), lr=cur)
            step += 1
        history.append(float(acc) / n_pairs)
        unet.status()                      # raises if a convolution's bounded wait gave up
        if log:
            log(f"epoch {ep + 1}/{epochs}: loss {history[-1]:.3e}")
        if on_epoch:
            on_epoch(ep, history)
    return history


def warm_start(net: unet.UNet3D, fdk: torch.Tensor, train_n: int | None = None) -> torch.Tensor:
    """The network's starting image for SIRT-TV from an FDK volume [n][n][n].

    train_n = None applies the network at the FDK's own resolution.  With
    train_n set (the training resolution), the FDK volume is averaged down to
    train_n^3, the network's correction (output - input) is computed there and
    added back after trilinear upsampling, so the network sees the voxel size
    it was trained on."""
    with torch.no_grad():
        if train_n is None or train_n == fdk.shape[-1]:
            return net.forward(fdk[None])[0]
        f = fdk.shape[-1] // train_n
        coarse = F.avg_pool3d(fdk[None, None], f)[0, 0].contiguous()
        corr = net.forward(coarse[None]) - coarse[None]
        up = F.interpolate(corr[None], scale_factor=f, mode="trilinear", align_corners=False)[0, 0]
        return (fdk + up).contiguous()


def save(net: unet.UNet3D, path: Path = WEIGHTS, **meta):
    path.parent.mkdir(parents=True, exist_ok=True)
    arrays = {k: v.detach().to(torch.bfloat16).view(torch.int16).cpu().numpy() for k, v in net.params.items()}
    np.savez_compressed(path, **arrays, meta=np.array(repr(meta)))


def load(path: Path = WEIGHTS, device="cuda") -> unet.UNet3D:
    """A UNet3D with the weights saved by ``save`` (stored as bf16)."""
    d = np.load(path)
    net = unet.UNet3D(seed=0, device=device)
    sd = {k: torch.from_numpy(d[k]).view(torch.bfloat16).float() for k in net.params}
    net.load_state_dict(sd)
    return net


def time_to_residual(result, tol: float, t_start: float = 0.0):
    """(iterations, seconds) until the relative data residual first reached tol,
    from a run whose per-iteration times are in result.times; None if never."""
    for (it, r), t in zip(result.residuals, result.times):
        if r <= tol:
            return it, t_start + t
    return None


def _main(argv=None):
    """python -m ctgb.warmstart --pairs 2000 --epochs 6 --out weights.npz: generate
    the training pairs, train, save the weights after every epoch, and compare
    plain and learned SIRT-TV on held-out phantoms at the training size."""
    import argparse
    ap = argparse.ArgumentParser(description=_main.__doc__)
    ap.add_argument("--pairs", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--views", type=int, default=90)
    ap.add_argument("--iters", type=int, default=500)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--seed0", type=int, default=1000)
    ap.add_argument("--holdout", type=int, default=4)
    ap.add_argument("--out", type=Path, default=WEIGHTS)
    ap.add_argument("--init", type=Path, default=None, help="start from these weights (fine-tuning)")
    ap.add_argument("--lr-end", type=float, default=3e-5)
    args = ap.parse_args(argv)

    def log(m):
        print(m, flush=True)

    from . import load as load_lib
    load_lib()
    t0 = time.perf_counter()
    pairs = generate(args.pairs, args.n, args.views, args.iters, args.seed0, log=log)
    log(f"generated {args.pairs} pairs in {pairs.seconds:.1f} s; target residual median "
        f"{float(np.median(pairs.residuals)):.3e}")
    net = load(args.init) if args.init else unet.UNet3D(seed=0)
    meta = dict(pairs=args.pairs, n=args.n, views=args.views, iters=args.iters, seed0=args.seed0,
                gen_seconds=round(pairs.seconds, 1), lr=args.lr, lr_end=args.lr_end)
    if args.init:
        meta["init"] = str(np.load(args.init)["meta"])

    def on_epoch(ep, hist):
        save(net, args.out, **meta, epochs_done=ep + 1, loss=[round(v, 8) for v in hist])

    tt = time.perf_counter()
    hist = train(net, pairs, epochs=args.epochs, lr=args.lr, lr_end=args.lr_end, log=log, on_epoch=on_epoch)
    meta["train_seconds"] = round(time.perf_counter() - tt, 1)
    del pairs
    torch.cuda.empty_cache()
    # held-out comparison at the training size
    plan = ConePlan(scan(args.n, args.views))
    loop = AsdLoop(plan, AsdConfig(iters=args.iters), use_graph=True)
    rows = []
    for k in range(args.holdout):
        vol = phantom_volume(args.n, 90000 + k)
        b = plan.fp(vol)
        fdk = plan.fdk(b)
        ref = loop.run(b, fdk, check_every=1)
        learned = warm_start(net, fdk)
        got = loop.run(b, learned, check_every=1)
        tol = ref.residuals[-1][1]
        hit = time_to_residual(got, tol)
        err = lambda a, c: float((a - c).norm() / c.norm())
        rows.append(dict(tol=tol, plain_iters=args.iters, learned_iters=None if hit is None else hit[0],
                         fdk_err=err(fdk, ref.x), start_err=err(learned, ref.x), final_err=err(got.x, ref.x)))
        log(f"held-out {k}: {rows[-1]}")
    meta["holdout"] = rows
    save(net, args.out, **meta, epochs_done=args.epochs, loss=[round(v, 8) for v in hist])
    log(f"done in {time.perf_counter() - t0:.1f} s")


if __name__ == "__main__":
    _main()
