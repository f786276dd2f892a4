"""Batched uneven 2D fan slices: one launch per operator reproduces the
single-slice operators exactly, and a graph-captured batched SIRT run equals
per-slice SIRT."""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _slices():
    from ctgb.geometry import fan_config
    from ctgb import phantom
    geoms = [fan_config(40, 30, 64, 200.0, 40.0), fan_config(57, 45, 90, 220.0, 57.0),
             fan_config(33, 18, 40, 150.0, 33.0), fan_config(64, 72, 101, 300.0, 64.0)]
    imgs = [phantom.ellipses_2d(g.nt, g.ns, phantom.ellipse_params(10, seed=20 + k)) for k, g in enumerate(geoms)]
    return geoms, imgs


def test_batched_operators_equal_single_slice():
    from ctgb.batch import FanBatch
    from ctgb.device import FanPlan
    geoms, imgs = _slices()
    batch = FanBatch(geoms)
    x = batch.pack_images(imgs)
    proj = batch.fp(x)
    back = batch.bp(proj)
    for k, g in enumerate(geoms):
        plan = FanPlan(g)
        p1 = plan.fp(imgs[k].cuda())
        assert torch.equal(batch.sino(proj, k), p1)
        assert torch.equal(batch.image(back, k), plan.bp(p1))
    # other block sizes: same numbers
    batch.set_blocks(64, 256)
    assert torch.equal(batch.fp(x), proj)
    assert torch.equal(batch.bp(proj), back)


def test_batched_fbp_equals_single_slice():
    from ctgb.batch import FanBatch
    from ctgb.device import FanPlan
    geoms, imgs = _slices()
    batch = FanBatch(geoms)
    proj = batch.fp(batch.pack_images(imgs))
    rec = batch.fbp(proj)
    for k, g in enumerate(geoms):
        assert torch.equal(batch.image(rec, k), FanPlan(g).fbp(batch.sino(proj, k).contiguous()))


def test_batched_sirt_graph_equals_per_slice_sirt():
    from ctgb.batch import FanBatch, BatchedSirt
    from ctgb.device import FanPlan
    from ctgb.sirt import Sirt, SirtConfig, MATLAB_EPS
    geoms, imgs = _slices()
    batch = FanBatch(geoms)
    b = batch.fp(batch.pack_images(imgs))
    x = torch.zeros(batch.n_img, dtype=torch.float32, device="cuda")
    hist = BatchedSirt(batch, b).run(x, 6, graph=True)
    assert hist.shape == (6, len(geoms))
    for k, g in enumerate(geoms):
        plan = FanPlan(g)
        res = Sirt(plan, batch.sino(b, k).contiguous(),
                   SirtConfig(iters=6, lam=2.0, lo=0.0, hi=1.0, eps=MATLAB_EPS)).run()
        assert torch.equal(batch.image(x, k), res.x)
        ref_r = np.array([r for _, r in res.residuals])
        assert np.allclose(hist[:, k], ref_r, rtol=1e-9)
        assert hist[-1, k] < hist[0, k]


def test_autotune_picks_a_candidate_and_caches(tmp_path, monkeypatch):
    from ctgb import batch as bmod
    monkeypatch.setattr(bmod, "_CACHE", tmp_path / "tune.json")
    geoms, imgs = _slices()
    batch = bmod.FanBatch(geoms)
    b = batch.fp(batch.pack_images(imgs))
    entry = bmod.autotune(batch, b, reps=1)
    fb, bb = entry["blocks"]
    assert fb in bmod.FP_BLOCKS and bb in bmod.BP_BLOCKS and batch.blocks == (fb, bb)
    assert len(entry["candidates"]) == len(bmod.FP_BLOCKS) * len(bmod.BP_BLOCKS)
    again = bmod.autotune(bmod.FanBatch(geoms), b)
    assert again["blocks"] == [fb, bb]
