"""Learned warm start for SIRT-TV (ctgb/warmstart.py) and the SIRT-TV loop it
feeds (ctgb/sirt.py: AsdLoop, the device-side ASD-POCS step ct_tv_flow_asd)."""
import math

import numpy as np
import pytest
import torch

from conftest import rel_l2


def test_training_scan_is_the_workload_scan_scaled():
    from ctgb import warmstart as ws
    g = ws.scan(128, 90)
    assert g.vol_shape == (128, 128, 128) and g.sino_shape == (90, 128, 192)
    assert tuple(g.size) == (200.0, 200.0, 150.0) and g.D == 600.0
    assert float(g.P[1] - g.P[0]) == pytest.approx(1.6, rel=1e-4)   # 3.2 mm at SDD 1200 -> 1.6 mm at the centre
    big = ws.scan(512, 90)
    assert big.sino_shape == (90, 512, 768)
    assert float(big.P[1] - big.P[0]) == pytest.approx(0.4, rel=1e-4)


def test_committed_weights_load():
    from ctgb import unet, warmstart as ws
    if not ws.WEIGHTS.exists():
        pytest.skip("no trained weights in the tree")
    net = ws.load(device="cpu")
    for name, cin, cout, taps, _ in unet.LAYERS:
        assert tuple(net.params[name + ".w"].shape) == (cout, taps, cin)
        assert torch.isfinite(net.params[name + ".w"]).all()
    assert float(net.params["head.w"].abs().sum()) > 0          # trained, not the identity start
    meta = str(np.load(ws.WEIGHTS)["meta"])
    assert "pairs" in meta and "epochs_done" in meta


@pytest.mark.gpu
def test_tv_flow_asd_is_the_host_composition():
    """The device ASD phase equals tv_flow with the host-computed step
    alpha * ||x - prev|| / sqrt(n), and updates alpha by its rule."""
    from ctgb import device as dev
    g = torch.Generator(device="cuda").manual_seed(3)
    prev = torch.rand((20, 24, 28), device="cuda", generator=g)
    x = (prev + 0.01 * torch.randn(prev.shape, device="cuda", generator=g)).clamp_(min=0)
    alpha = 0.3
    dp = float(torch.linalg.vector_norm((x - prev).double()))
    ref = x.clone()
    dev.tv_flow(ref, 5, alpha * dp / math.sqrt(x.numel()), 1e-8, 0.0)
    got, p2 = x.clone(), prev.clone()
    work = torch.empty_like(x)
    scratch = torch.zeros(2, dtype=torch.float64, device="cuda")
    state = torch.tensor([alpha, 0.0, 0.0], dtype=torch.float64, device="cuda")
    dev.tv_flow_asd(got, p2, work, scratch, state, 5, 1e-8, 0.0, 0.5, 0.95)
    torch.cuda.synchronize()
    assert torch.equal(p2, x)                                      # prev now holds x after the data step
    assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-6
    assert float(state[1]) == pytest.approx(dp * dp, rel=1e-9)
    dg = float(torch.linalg.vector_norm((got - x).double()))
    assert float(state[2]) == pytest.approx(dg * dg, rel=1e-6)
    assert float(state[0]) == pytest.approx(alpha * (0.5 if dg > 0.95 * dp else 1.0))


@pytest.mark.gpu
def test_asd_loop_graph_replays_eager_and_reduces_the_residual():
    from ctgb import warmstart as ws
    from ctgb.device import ConePlan
    from ctgb.sirt import AsdConfig, AsdLoop
    plan = ConePlan(ws.scan(64, 30))
    vol = ws.phantom_volume(64, 11)
    b = plan.fp(vol)
    fdk = plan.fdk(b)
    cfg = AsdConfig(iters=25)
    eager = AsdLoop(plan, cfg).run(b, fdk, check_every=1)
    loop = AsdLoop(plan, cfg, use_graph=True)
    graph = loop.run(b, fdk, check_every=5)
    assert torch.equal(eager.x, graph.x) and eager.alpha == graph.alpha
    again = loop.run(b, fdk, check_every=25)                      # a second run restarts cleanly
    assert torch.equal(again.x, graph.x)
    r = [v for _, v in eager.residuals]
    assert r[-1] < 0.5 * r[0]
    # the residual norms are sums of FP64 atomics: equal between runs up to the last bits
    tol = r[10] * (1 + 1e-6)
    assert r[9] > tol
    stop = AsdLoop(plan, cfg).run(b, fdk, tol=tol, check_every=1)
    assert stop.iterations == 11 and ws.time_to_residual(stop, tol)[0] == 11


@pytest.mark.gpu
def test_untrained_network_start_is_the_fdk_volume():
    from ctgb import unet, warmstart as ws
    net = unet.UNet3D(seed=0)                                      # zero head: identity
    fdk = torch.rand((128, 128, 128), device="cuda")
    assert torch.equal(ws.warm_start(net, fdk), fdk)
    assert rel_l2(ws.warm_start(net, fdk, train_n=64).cpu().numpy(), fdk.cpu().numpy()) <= 1e-6


def test_weights_round_trip_through_save_and_load(tmp_path):
    """save() stores bf16 weights with their metadata; load() (also used to
    fine-tune from saved weights) restores them."""
    from ctgb import unet, warmstart as ws
    net = unet.UNet3D(seed=5, device="cpu")
    g = torch.Generator().manual_seed(1)
    net.params["head.w"] = torch.randn(32, generator=g)
    path = tmp_path / "w.npz"
    ws.save(net, path, pairs=3, note="test")
    back = ws.load(path, device="cpu")
    for k, v in net.params.items():
        assert torch.equal(back.params[k], v.to(torch.bfloat16).float()), k
    assert "note" in str(np.load(path)["meta"])


def test_time_to_residual_reads_the_first_check_at_or_below_tol():
    from types import SimpleNamespace
    from ctgb import warmstart as ws
    run = SimpleNamespace(residuals=[(1, 0.3), (2, 0.2), (3, 0.1), (4, 0.05)], times=[0.5, 1.0, 1.5, 2.0])
    assert ws.time_to_residual(run, 0.1) == (3, 1.5)
    assert ws.time_to_residual(run, 0.1, t_start=0.25) == (3, 1.75)
    assert ws.time_to_residual(run, 0.01) is None


def test_flip_augmentations_map_the_view_set_as_documented():
    """x / y flips of the volume map the source angle b to -b / pi - b and keep
    the 90-view set; the x-y swap maps b to 3 pi / 2 - b, the set turned by half
    a view step."""
    from ctgb import warmstart as ws
    g = ws.scan(128, 90)
    deg = np.round(np.degrees(g.beta.astype(np.float64)), 3) % 360.0     # float32 angles, to 0.001 degree
    base = set(deg)
    assert len(base) == 90 and all(d % 4 == 0 for d in deg)

    def mapped(f):
        return set(np.round(f(deg), 3) % 360.0)

    assert mapped(lambda b: -b) == base                      # x flip: source (C_t - D sin b) mirrored
    assert mapped(lambda b: 180.0 - b) == base               # y flip: source (C_s + D cos b) mirrored
    swapped = mapped(lambda b: 270.0 - b)                    # x-y swap
    assert swapped == set(np.round(deg + 2.0, 3) % 360.0)
    # the mirrored source positions are those of the mapped angles
    b = np.radians(deg)
    for f, sx, sy in ((lambda v: -v, -1, 1), (lambda v: np.pi - v, 1, -1)):
        assert np.allclose(sx * -np.sin(b), -np.sin(f(b))) and np.allclose(sy * np.cos(b), np.cos(f(b)))
    assert np.allclose(np.cos(b), -np.sin(1.5 * np.pi - b)) and np.allclose(-np.sin(b), np.cos(1.5 * np.pi - b))
