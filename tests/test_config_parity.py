"""Parity at the benchmark workloads' own sizes, against the oracle.

* the 512^3 / 768x512 backprojector (the bench's dominant kernel) on views of
  the bench scan;
* FDK of the 256^3 / 360-view / 512x384 scan on a view subset, in both filter
  and backprojection modes (FDK.cu:129-611);
* the 2D fan FP + FBP scan in full: 256^2, 360 views, 512 bins, Shepp-Logan
  (the reference's filter, launch-order pre-weight) and Ram-Lak;
* the largest and smallest slices of the batched 2D SIRT workload (512^2 /
  720 views / 1024 bins, 128^2 / 90 / 256) through the batch operators: FP, BP
  and 6 SIRT iterations against the FP64 oracle loop.

Tolerances: rel-L2 <= 1e-5 for single operators (FP32 against the reference's
FP64 arithmetic); 1e-4 after 6 SIRT iterations (FP32 accumulated).
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def test_bp_512_views_vs_oracle(oracle):
    import torch
    from ctgb.device import ConePlan
    from ctgb.geometry import config_cone_512
    geom = config_cone_512().subset_views([17, 133])
    g = torch.Generator(device="cuda").manual_seed(5)
    sino = torch.rand(geom.sino_shape, device="cuda", generator=g)
    out = ConePlan(geom).bp(sino).cpu().numpy()
    ref = oracle.cone_bp(sino.cpu().numpy(), geom.beta, geom.P, geom.xi, geom.size, geom.D, geom.vol_shape)
    assert rel_l2(out, ref) <= TOL


@pytest.mark.parametrize("filter_mode,bp_mode", [(1, 1), (0, 0)])
def test_fdk_256_view_subset_vs_oracle(oracle, filter_mode, bp_mode):
    import torch
    from ctgb.device import ConePlan
    from ctgb.geometry import config_cone_fdk
    from ctgb import phantom
    full = config_cone_fdk()
    geom = full.subset_views(np.arange(0, 360, 30))           # 12 of the 360 views, full detector
    vol = phantom.ellipsoids_3d(geom.nt, geom.ns, geom.nz, phantom.ellipsoid_params(12, seed=1), device="cuda")
    plan = ConePlan(geom, fdk_filter=filter_mode, fdk_bp=bp_mode)
    proj = plan.fp(vol)
    out = plan.fdk(proj).cpu().numpy()
    ref = oracle.fdk(proj.cpu().numpy(), geom.beta, geom.P, geom.xi, geom.size, geom.D, geom.vol_shape,
                     filter_mode=filter_mode, sticky=bp_mode)
    assert rel_l2(out, ref) <= TOL


def test_fan_config_full_fp_and_fbp_vs_oracle(oracle):
    import torch
    from ctgb.device import FanPlan
    from ctgb.geometry import config_fan2d
    from ctgb import phantom
    geom = config_fan2d()
    assert (geom.nt, len(geom.beta), len(geom.P)) == (256, 360, 512)
    img = phantom.ellipses_2d(256, 256, phantom.ellipse_params(10, seed=0)).numpy()
    plan = FanPlan(geom)
    proj = plan.fp(torch.from_numpy(img).cuda())
    ref = oracle.fan_fp(img, geom.beta, geom.P, geom.size, geom.D)
    assert rel_l2(proj.cpu().numpy(), ref) <= TOL
    sino = ref.astype(np.float32)
    b32, p32 = geom.beta.astype(np.float32), geom.P.astype(np.float32)
    d_sino = torch.from_numpy(sino).cuda()
    out = plan.fbp(d_sino, filter_mode=1).cpu().numpy()                # Shepp-Logan, reference launch order
    refi = oracle.fbpfan(sino, b32, p32, geom.size, geom.img_shape, geom.D, filter_mode=1)
    assert rel_l2(out, refi) <= TOL
    plan.set_filter("ram-lak")
    out = plan.fbp(d_sino, filter_mode=0).cpu().numpy()
    rc = oracle.fbpfan_filter_ex(sino, b32, p32, geom.D, mode=0, kind=1)
    refi = oracle.fbpfan_bp(rc, b32, p32, geom.size, geom.img_shape, geom.D)
    assert rel_l2(out, refi) <= TOL
    # the FBP reconstructs the phantom (a property of the method, not of the port)
    disc = np.hypot(*np.mgrid[:256, :256] - 127.5) < 0.45 * 256
    assert np.linalg.norm((out - img)[disc]) / np.linalg.norm(img[disc]) < 0.25


def test_batch_extreme_slices_vs_oracle(oracle):
    import torch
    from ctgb.batch import FanBatch, BatchedSirt
    from ctgb.geometry import fan_config
    from ctgb.sirt import MATLAB_EPS
    from ctgb import phantom
    from oracle.oracle import sirt_loop
    geoms = [fan_config(512, 720, 1024, 500.0, 512.0), fan_config(128, 90, 256, 500.0, 128.0)]
    imgs = [phantom.ellipses_2d(g.nt, g.ns, phantom.ellipse_params(10, seed=60 + k)).numpy()
            for k, g in enumerate(geoms)]
    batch = FanBatch(geoms)
    sinos = [oracle.fan_fp(im, g.beta, g.P, g.size, g.D) for g, im in zip(geoms, imgs)]
    proj = batch.fp(batch.pack_images(imgs))
    b = batch.pack_sinos([s.astype(np.float32) for s in sinos])
    back = batch.bp(b)
    for k, g in enumerate(geoms):
        assert rel_l2(batch.sino(proj, k).cpu().numpy(), sinos[k]) <= TOL, k
        refb = oracle.fan_bp(sinos[k].astype(np.float32), g.beta.astype(np.float32), g.P.astype(np.float32),
                             g.size, g.img_shape, g.D)
        assert rel_l2(batch.image(back, k).cpu().numpy(), refb) <= TOL, k
    x = torch.zeros(batch.n_img, dtype=torch.float32, device="cuda")
    BatchedSirt(batch, b).run(x, 6, graph=True)
    for k, g in enumerate(geoms):
        b32, p32 = g.beta.astype(np.float32), g.P.astype(np.float32)
        fp = lambda v, g=g: oracle.fan_fp(v.astype(np.float32), g.beta, g.P, g.size, g.D)
        bp = lambda y, g=g, b32=b32, p32=p32: oracle.fan_bp(y.astype(np.float32), b32, p32, g.size, g.img_shape, g.D)
        ref = sirt_loop(fp, bp, sinos[k].astype(np.float32), np.zeros(g.img_shape), 6, 2.0, 0.0, 1.0, MATLAB_EPS)
        assert rel_l2(batch.image(x, k).cpu().numpy(), ref) <= 1e-4, k
