"""Filter family on the GPU: Ram-Lak taps, Hamming smoothing window and
short-scan (Parker) weights in the FDK and fan FBP filter stages, against the
oracle's restatement (rel-L2 <= 1e-5, FP32)."""
import math

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5

OPTIONS = [("ram-lak", 0, False), ("shepp-logan", 15, False), ("ram-lak", 10, True), ("shepp-logan", 0, True)]


def _kind(name):
    return {"shepp-logan": 0, "ram-lak": 1}[name]


def _short_fan(n=48, nbins=150, D=150.0, seed=7):
    from ctgb import phantom
    from ctgb.geometry import FanGeometry
    maxp = 1.1 * n * math.sqrt(2) / 2
    P = np.linspace(-maxp, maxp, nbins)
    fan = abs(math.atan(P[-1] / D) - math.atan(P[0] / D))
    db = 2 * math.pi / 360
    beta = np.arange(int(math.ceil((math.pi + fan) / db)) + 1) * db
    geom = FanGeometry(n, n, (float(n), float(n)), beta, P, D)
    img = phantom.ellipses_2d(n, n, phantom.ellipse_params(10, seed=seed)).numpy()
    return geom, img


@pytest.mark.parametrize("kind,window,short", OPTIONS)
def test_fdk_filter_options_match_oracle(golden, oracle, kind, window, short):
    import torch
    from ctgb.device import ConePlan, FDK_FILTER_CLEAN, FDK_FILTER_LAUNCH_ORDER
    from ctgb.geometry import ConeGeometry
    P, xi, beta = golden["fdk_P"], golden["fdk_xi"], golden["fdk_beta"]
    size, D = golden["fdk_size"], float(golden["fdk_D"])
    geom = ConeGeometry(16, 16, 14, size, beta, P, xi, D)
    proj = golden["fdk_proj"]
    for mode in (FDK_FILTER_CLEAN, FDK_FILTER_LAUNCH_ORDER):
        plan = ConePlan(geom, fdk_filter=mode).set_filter(kind, window, short)
        out = plan.fdk_filter(torch.from_numpy(proj).cuda()).cpu().numpy()
        ref = oracle.fdk_filter_ex(proj, beta, P, xi, D, mode=mode, kind=_kind(kind), window=window,
                                   short_scan=short)
        assert rel_l2(out, ref) <= TOL, (mode, kind, window, short)


@pytest.mark.parametrize("kind,window,short", OPTIONS)
def test_fan_fbp_options_match_oracle(oracle, kind, window, short):
    import torch
    from ctgb.device import FanPlan
    geom, img = _short_fan()
    sino = oracle.fan_fp(img, geom.beta, geom.P, geom.size, geom.D).astype(np.float32)
    b32, p32 = geom.beta.astype(np.float32), geom.P.astype(np.float32)
    plan = FanPlan(geom).set_filter(kind, window, short)
    for mode in (0, 1):
        out = plan.fbp(torch.from_numpy(sino).cuda(), filter_mode=mode).cpu().numpy()
        rc = oracle.fbpfan_filter_ex(sino, b32, p32, geom.D, mode=mode, kind=_kind(kind), window=window,
                                     short_scan=short)
        ref = oracle.fbpfan_bp(rc, b32, p32, geom.size, (geom.ns, geom.nt), geom.D)
        assert rel_l2(out, ref) <= TOL, (mode, kind, window, short)


def test_short_scan_fbp_reconstructs_like_a_full_scan():
    """On the GPU: Parker-weighted FBP over pi + fan angle keeps the image
    scale and error of a full-turn FBP of the same object."""
    import torch
    from ctgb.device import FanPlan
    from ctgb.geometry import FanGeometry
    geom, img = _short_fan(n=96, nbins=256, D=250.0, seed=9)
    full = FanGeometry(geom.nt, geom.ns, geom.size, np.arange(360) * (2 * math.pi / 360), geom.P, geom.D)
    x = torch.from_numpy(img).cuda()
    yy, xx = np.mgrid[:96, :96]
    disc = (yy - 47.5) ** 2 + (xx - 47.5) ** 2 < (0.45 * 96) ** 2

    def err(g, short):
        plan = FanPlan(g).set_filter("shepp-logan", 0, short)
        rec = plan.fbp(plan.fp(x), filter_mode=0).cpu().numpy()
        return np.linalg.norm((rec - img)[disc]) / np.linalg.norm(img[disc]), rec[disc].mean() / img[disc].mean()

    e_full, m_full = err(full, False)
    e_short, m_short = err(geom, True)
    assert abs(m_short - 1) < 0.01 and abs(m_full - 1) < 0.01
    assert e_short < 1.2 * e_full + 0.01


def test_reference_defaults_unchanged_by_resetting(golden, oracle):
    """Setting the options back to the defaults gives the reference filter again."""
    import torch
    from ctgb.device import ConePlan
    from ctgb.geometry import ConeGeometry
    P, xi, beta = golden["fdk_P"], golden["fdk_xi"], golden["fdk_beta"]
    geom = ConeGeometry(16, 16, 14, golden["fdk_size"], beta, P, xi, float(golden["fdk_D"]))
    plan = ConePlan(geom)
    proj = torch.from_numpy(golden["fdk_proj"]).cuda()
    base = plan.fdk_filter(proj).cpu().numpy()
    plan.set_filter("ram-lak", 15, True)
    assert rel_l2(plan.fdk_filter(proj).cpu().numpy(), base) > 1e-3
    plan.set_filter()
    np.testing.assert_array_equal(plan.fdk_filter(proj).cpu().numpy(), base)


def test_batch_filter_options_match_single_plans(oracle):
    import torch
    from ctgb.batch import FanBatch
    from ctgb.device import FanPlan
    g1, img1 = _short_fan(n=40, nbins=120, D=140.0, seed=3)
    g2, img2 = _short_fan(n=56, nbins=170, D=170.0, seed=4)
    batch = FanBatch([g1, g2]).set_filter("ram-lak", 15, True)
    sinos = [oracle.fan_fp(im, g.beta, g.P, g.size, g.D).astype(np.float32) for g, im in ((g1, img1), (g2, img2))]
    packed = torch.from_numpy(np.concatenate([s.ravel() for s in sinos])).cuda()
    out = torch.zeros(batch.n_img, dtype=torch.float32, device="cuda")
    batch.fbp(packed, out, filter_mode=1)
    for k, (g, s) in enumerate(zip((g1, g2), sinos)):
        ref = FanPlan(g).set_filter("ram-lak", 15, True).fbp(torch.from_numpy(s).cuda(), filter_mode=1)
        got = out[int(batch.img_off[k]):int(batch.img_off[k + 1])].view(g.ns, g.nt)
        assert torch.equal(got, ref)
