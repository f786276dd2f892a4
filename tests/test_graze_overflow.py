"""Rays along a grid plane: every one of them gets the reference's FP64 walk.

The reference clamps the slopes of a ray that runs along a t, s or z plane at
1e16 and charges its segments by the rounding of that walk
(ProjectionCone_3D.cu:44-84, ProjectionFan_2D.cu:37-49).  The fast projectors
list such rays for an FP64 re-walk; past the list's capacity they set a bit
per ray that the re-walk drains.  These tests make more grazing rays than the
list holds and check the projections against the oracle, and the fused
residual norms (where the fast kernel leaves grazing rays out and the re-walk
adds them) against the unfused composition.

Tolerances: rel-L2 <= 1e-5 against the oracle (FP32 against the reference's
FP64 arithmetic); 1e-6 relative on the norms; exact equality between runs.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5
CAP = 1 << 16


@pytest.fixture
def torch_cuda():
    import torch
    from ctgb.device import set_graze_list_capacity
    yield torch
    set_graze_list_capacity(CAP)


def _central_row_cone():
    """64^3 volume (even z count: the rotation plane z = 32 is a grid plane),
    360 views, 256 bins and 65 rows whose centre row sits 1e-6 mm off that
    plane, as a detector domain computed in floating point can.  Every hit ray
    of the centre row grazes: 360 x ~250 > 65536."""
    from ctgb.geometry import ConeGeometry, view_angles, centred_domain
    from ctgb import phantom
    xi = centred_domain(65, 0.4) + 1e-6
    geom = ConeGeometry(64, 64, 64, (64.0, 64.0, 64.0), view_angles(360), centred_domain(256, 0.35), xi, 200.0)
    vol = phantom.ellipsoids_3d(64, 64, 64, phantom.ellipsoid_params(12, seed=31)).numpy()
    return geom, vol


def test_cone_grazing_rays_beyond_list_capacity(oracle, torch_cuda):
    from ctgb.device import ConePlan
    torch = torch_cuda
    geom, vol = _central_row_cone()
    plan = ConePlan(geom)
    x = torch.from_numpy(vol).cuda()
    proj = plan.fp(x)
    n = plan.grazing_rays()
    assert n > CAP, n
    ref = oracle.cone_fp(vol, geom.beta, geom.P, geom.xi, geom.size, geom.D)
    got = proj.cpu().numpy()
    assert rel_l2(got, ref) <= TOL
    assert rel_l2(got[:, 32, :], ref[:, 32, :]) <= TOL      # the grazing row on its own
    # the overflow map is drained: a second projection is identical
    assert torch.equal(plan.fp(x), proj)
    assert plan.grazing_rays() == n
    # residual mode: the norm includes every grazing ray
    b = proj * 1.01 + 0.001
    rowsum = plan.fp(torch.ones_like(x))
    out, norms = plan.fp_residual(x, b, rowsum, 1e-6)
    r = (b - proj).double()
    assert abs(norms[0].item() - (r * r).sum().item()) <= 1e-6 * (r * r).sum().item()
    assert rel_l2(out.cpu().numpy(), ((b - proj) / (rowsum + 1e-6)).cpu().numpy()) <= 1e-6


def test_cone_result_does_not_depend_on_list_capacity(torch_cuda):
    from ctgb.device import ConePlan, set_graze_list_capacity
    torch = torch_cuda
    geom, vol = _central_row_cone()
    geom = geom.subset_views(np.arange(0, 360, 8))
    x = torch.from_numpy(vol).cuda()
    full = ConePlan(geom).fp(x)
    for cap in (1, 1000):
        set_graze_list_capacity(cap)
        plan = ConePlan(geom)
        assert torch.equal(plan.fp(x), full), cap
        b = full + 0.5
        _, norms = plan.fp_residual(x, b)
        r = (b - full).double()
        assert abs(norms[0].item() - (r * r).sum().item()) <= 1e-6 * (r * r).sum().item()


def _axis_fan():
    """128^2 fan scan whose views include the four axis angles, with an odd
    detector: the centre ray of each axis view runs along a grid line."""
    from ctgb.geometry import FanGeometry, view_angles, centred_domain
    return FanGeometry(128, 128, (128.0, 128.0), view_angles(360), centred_domain(255, 0.5), 300.0)


def test_fan_grazing_overflow_matches_oracle(oracle, torch_cuda):
    from ctgb.device import FanPlan, set_graze_list_capacity
    from ctgb import phantom
    torch = torch_cuda
    geom = _axis_fan()
    img = phantom.ellipses_2d(128, 128, phantom.ellipse_params(10, seed=5)).numpy()
    x = torch.from_numpy(img).cuda()
    full = FanPlan(geom).fp(x)
    set_graze_list_capacity(1)
    plan = FanPlan(geom)
    proj = plan.fp(x)
    assert plan.grazing_rays() >= 2
    assert torch.equal(proj, full)
    ref = oracle.fan_fp(img, geom.beta, geom.P, geom.size, geom.D)
    assert rel_l2(proj.cpu().numpy(), ref) <= TOL
    b = proj + 0.25
    _, norms = plan.fp_residual(x, b)
    r = (b - proj).double()
    assert abs(norms[0].item() - (r * r).sum().item()) <= 1e-6 * (r * r).sum().item()


def test_batch_grazing_overflow_matches_single_slices(oracle, torch_cuda):
    from ctgb.batch import FanBatch
    from ctgb.device import FanPlan, set_graze_list_capacity
    from ctgb.geometry import fan_config
    from ctgb import phantom
    torch = torch_cuda
    geoms = [fan_config(96, 120, 200, 500.0), _axis_fan(), fan_config(64, 90, 130, 500.0)]
    imgs = [phantom.ellipses_2d(g.nt, g.ns, phantom.ellipse_params(10, seed=40 + k)).numpy()
            for k, g in enumerate(geoms)]
    set_graze_list_capacity(1)
    batch = FanBatch(geoms)
    x = batch.pack_images(imgs)
    proj = batch.fp(x)
    assert batch.grazing_rays() >= 2
    b = proj + 0.25
    out = torch.empty_like(b)
    norms = torch.zeros(2 * len(geoms), dtype=torch.float64, device="cuda")
    batch.fp_residual(x, b, None, 0.0, out, norms)
    for k, g in enumerate(geoms):
        single = FanPlan(g).fp(torch.from_numpy(imgs[k]).cuda())
        assert torch.equal(batch.sino(proj, k), single), k
        ref = oracle.fan_fp(imgs[k], g.beta, g.P, g.size, g.D)
        assert rel_l2(batch.sino(proj, k).cpu().numpy(), ref) <= TOL
        r = (batch.sino(b, k) - single).double()
        assert abs(norms[2 * k].item() - (r * r).sum().item()) <= 1e-6 * (r * r).sum().item()
