"""CUDA path (libctgb through its C ABI) against the oracle and the reference fixtures.

Tolerances: rel-L2 <= 1e-5 in FP32 against the reference arithmetic (the
FP64 oracle and the fixtures made by the reference kernels).
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    return torch


def _cone(golden, k):
    g = {n: golden[f"cone_{k}_{n}"] for n in ("vol", "proj", "R", "bp", "P", "xi", "beta", "size", "D")}
    g["D"] = float(g["D"])
    return g


@pytest.mark.parametrize("case", ["a", "b", "c"])
def test_cone_fp_dropin_matches_reference(golden, case):
    from ctgb import ops
    g = _cone(golden, case)
    nz, ns, nt = g["vol"].shape
    out = ops.ProjectionCone_3D(g["vol"].ravel(), nt, ns, nz, g["size"], g["beta"], g["P"], g["xi"], g["D"])
    assert out.dtype == np.float64 and out.shape == (g["proj"].size,)
    assert rel_l2(out, g["proj"].ravel()) <= TOL


@pytest.mark.parametrize("case", ["a", "b", "c"])
def test_cone_bp_dropin_matches_reference(golden, case):
    from ctgb import ops
    g = _cone(golden, case)
    nz, ns, nt = g["vol"].shape
    out = ops.Backprojection3D(g["R"].ravel(), g["xi"], g["P"], g["beta"], g["D"], g["size"], nt, ns, nz)
    assert rel_l2(out, g["bp"].ravel()) <= TOL


def _geom(g):
    from ctgb.geometry import ConeGeometry
    nz, ns, nt = g["vol"].shape
    return ConeGeometry(nt, ns, nz, g["size"], g["beta"], g["P"], g["xi"], g["D"])


@pytest.mark.parametrize("case", ["a", "b"])
def test_cone_device_plan_matches_reference(golden, torch_cuda, case):
    from ctgb.device import ConePlan
    torch = torch_cuda
    g = _cone(golden, case)
    plan = ConePlan(_geom(g))
    proj = plan.fp(torch.from_numpy(g["vol"]).cuda())
    assert rel_l2(proj.cpu().numpy(), g["proj"]) <= TOL
    bp = plan.bp(torch.from_numpy(g["R"]).cuda())
    assert rel_l2(bp.cpu().numpy(), g["bp"]) <= TOL


def _fdk_geom(golden):
    from ctgb.geometry import ConeGeometry
    return ConeGeometry(16, 16, 14, golden["fdk_size"], golden["fdk_beta"], golden["fdk_P"], golden["fdk_xi"],
                        float(golden["fdk_D"]))


def test_fdk_filter_stage_matches_reference(golden, oracle, torch_cuda):
    from ctgb.device import ConePlan, FDK_FILTER_CLEAN, FDK_FILTER_LAUNCH_ORDER
    torch = torch_cuda
    geom = _fdk_geom(golden)
    proj = torch.from_numpy(golden["fdk_proj"]).cuda()
    out = ConePlan(geom, fdk_filter=FDK_FILTER_CLEAN).fdk_filter(proj).cpu().numpy()
    assert rel_l2(out, golden["fdk_conv"]) <= TOL
    out = ConePlan(geom, fdk_filter=FDK_FILTER_LAUNCH_ORDER).fdk_filter(proj).cpu().numpy()
    ref = oracle.fdk_filter(golden["fdk_proj"], geom.P, geom.xi, geom.D, mode=1)
    assert rel_l2(out, ref) <= TOL


def test_fdk_bp_stage_matches_reference(golden, oracle, torch_cuda):
    from ctgb.device import ConePlan, FDK_BP_STICKY, FDK_BP_ZERO
    torch = torch_cuda
    geom = _fdk_geom(golden)
    conv = torch.from_numpy(golden["fdk_conv"]).cuda()
    out = ConePlan(geom, fdk_bp=FDK_BP_STICKY).fdk_bp(conv).cpu().numpy()
    assert rel_l2(out, golden["fdk_bp"]) <= TOL
    out = ConePlan(geom, fdk_bp=FDK_BP_ZERO).fdk_bp(conv).cpu().numpy()
    ref = oracle.fdk_bp(golden["fdk_conv"], geom.beta, geom.P, geom.xi, geom.size, geom.D, geom.vol_shape, sticky=0)
    assert rel_l2(out, ref) <= TOL


def test_fdk_matches_oracle_both_modes(golden, oracle, torch_cuda):
    from ctgb.device import ConePlan, FDK_FILTER_CLEAN, FDK_FILTER_LAUNCH_ORDER, FDK_BP_STICKY, FDK_BP_ZERO
    from ctgb.geometry import ConeGeometry
    torch = torch_cuda
    P, xi, beta = golden["fdk_P"], golden["fdk_xi"], golden["fdk_beta"]
    size, D = golden["fdk_size"], float(golden["fdk_D"])
    proj = golden["fdk_proj"]
    geom = ConeGeometry(16, 16, 14, size, beta, P, xi, D)
    for fmode, bmode in [(FDK_FILTER_LAUNCH_ORDER, FDK_BP_STICKY), (FDK_FILTER_CLEAN, FDK_BP_STICKY),
                         (FDK_FILTER_CLEAN, FDK_BP_ZERO)]:
        plan = ConePlan(geom, fdk_filter=fmode, fdk_bp=bmode)
        out = plan.fdk(torch.from_numpy(proj).cuda()).cpu().numpy()
        ref = oracle.fdk(proj, beta, P, xi, size, D, (14, 16, 16), filter_mode=fmode, sticky=bmode)
        assert rel_l2(out, ref) <= TOL, (fmode, bmode)
    # clean filter + sticky backprojection is the race-free reference chain
    plan = ConePlan(geom, fdk_filter=FDK_FILTER_CLEAN, fdk_bp=FDK_BP_STICKY)
    out = plan.fdk(torch.from_numpy(proj).cuda()).cpu().numpy()
    assert rel_l2(out, golden["fdk_bp"]) <= TOL


def test_fdk_dropin_matches_oracle(golden, oracle):
    from ctgb import ops
    P, xi, beta = golden["fdk_P"], golden["fdk_xi"], golden["fdk_beta"]
    size, D = golden["fdk_size"], float(golden["fdk_D"])
    proj = golden["fdk_proj"]
    out = ops.FDK(proj.ravel(), xi, P, beta, D, size, 16, 16, 14)
    ref = oracle.fdk(proj, beta, P, xi, size, D, (14, 16, 16), filter_mode=1, sticky=1)
    assert rel_l2(out, ref.ravel()) <= TOL


def test_fan_parallel_fp_dropin_match_reference(golden):
    from ctgb import ops
    img, size = golden["f2_img"], golden["f2_size"]
    beta, P = golden["f2_beta"], golden["f2_P"]
    ns, nt = img.shape
    assert rel_l2(ops.ProjectionFan_2D(img.ravel(), nt, ns, size, beta, P, 80.0), golden["f2_fp"].ravel()) <= TOL
    assert rel_l2(ops.ProjectionFan_2D(img.ravel(), nt, ns, size, beta, golden["f2_P_wide"], 80.0),
                  golden["f2_fp_wide"].ravel()) <= TOL
    # ProjectionParallel_2D(pic, height, width, Size, ...): the fixture image is [height=30][width=32]
    assert rel_l2(ops.ProjectionParallel_2D(img.ravel(), ns, nt, size, beta, P), golden["f2_par"].ravel()) <= TOL


def test_parallel_fp_matches_oracle(oracle, golden):
    from ctgb import ops
    img = golden["f2_img"]
    h, w = img.shape
    size = np.array([30.0, 32.0])          # Size = [height extent, width extent]
    beta, P = golden["f2_beta"], golden["f2_P"]
    ref = oracle.par_fp(img, beta, P, size)
    out = ops.ProjectionParallel_2D(img.ravel(), h, w, size, beta, P)
    assert rel_l2(out, ref.ravel()) <= TOL


def test_fan_bp_fbp_dropin_match_reference(golden):
    from ctgb import ops
    size = golden["f2_size"]
    out = ops.BackprojectionFan2D(golden["f2_fp"].astype(np.float32).ravel(), golden["f2_beta"], golden["f2_P"],
                                  size, 32, 30, 80.0)
    assert rel_l2(out, golden["f2_bp"].ravel()) <= TOL
    out = ops.FBPparallel(golden["f2_par"].astype(np.float32).ravel(), golden["f2_beta"], golden["f2_P"], size, 32, 30)
    assert rel_l2(out, golden["f2_fbppar"].ravel()) <= TOL


def test_fbpfan_matches_oracle(golden, oracle):
    from ctgb import ops
    size, P, beta = golden["f2_size"], golden["f2_P150"], golden["f2_beta20"]
    sino = golden["f2_sino150"]
    out = ops.FBPfan(sino.ravel(), beta, P, size, 32, 30, 80.0)
    ref = oracle.fbpfan(sino, beta, P, size, (30, 32), 80.0, filter_mode=1)
    assert rel_l2(out, ref.ravel()) <= TOL


def _random_cone(seed, shape=(40, 44, 48), nb=24, np_=64, nx=48):
    from ctgb.geometry import ConeGeometry, view_angles, centred_domain
    from ctgb import phantom
    nz, ns, nt = shape
    size = (nt * 0.5, ns * 0.5, nz * 0.5)
    geom = ConeGeometry(nt, ns, nz, size, view_angles(nb), centred_domain(np_, 0.45), centred_domain(nx, 0.42), 70.0)
    vol = phantom.ellipsoids_3d(nt, ns, nz, phantom.ellipsoid_params(12, seed=seed)).numpy()
    return geom, vol


def test_cone_fp_bp_medium_vs_oracle(oracle, torch_cuda):
    from ctgb.device import ConePlan
    torch = torch_cuda
    geom, vol = _random_cone(21)
    plan = ConePlan(geom)
    proj = plan.fp(torch.from_numpy(vol).cuda()).cpu().numpy()
    ref = oracle.cone_fp(vol, geom.beta, geom.P, geom.xi, geom.size, geom.D)
    assert rel_l2(proj, ref) <= TOL
    bp = plan.bp(torch.from_numpy(ref).cuda()).cpu().numpy()
    refbp = oracle.cone_bp(ref, geom.beta, geom.P, geom.xi, geom.size, geom.D, geom.vol_shape)
    assert rel_l2(bp, refbp) <= TOL


def test_cone_segment_count_exact(oracle):
    from ctgb.device import ConePlan
    from ctgb.geometry import config_cone_fdk
    geom = config_cone_fdk().with_views(36)
    n_gpu = ConePlan(geom).count_segments()
    n_cpu = oracle.cone_segments(geom.vol_shape, geom.size, geom.beta, geom.P, geom.xi, geom.D)
    # the count is exact up to FP64 rounding of rays that touch a box edge
    assert abs(n_gpu - n_cpu) <= 1e-6 * n_cpu


def test_full_size_fp_subset_vs_oracle(oracle, torch_cuda):
    """512^3, 768x512 detector: two views checked ray by ray against the oracle."""
    from ctgb.device import ConePlan
    from ctgb.geometry import config_cone_512
    from ctgb import phantom
    torch = torch_cuda
    geom = config_cone_512().subset_views([44, 200])
    vol = phantom.ellipsoids_3d(geom.nt, geom.ns, geom.nz, phantom.ellipsoid_params(12, seed=2), device="cuda")
    proj = ConePlan(geom).fp(vol).cpu().numpy()
    ref = oracle.cone_fp(vol.cpu().numpy(), geom.beta, geom.P, geom.xi, geom.size, geom.D)
    assert rel_l2(proj, ref) <= TOL


def test_fp_of_constant_volume_is_chord_length(torch_cuda):
    """A(1) = length of each ray inside the box (512^3 geometry, 8 views)."""
    from ctgb.device import ConePlan
    from ctgb.geometry import config_cone_512
    torch = torch_cuda
    geom = config_cone_512().with_views(8)
    ones = torch.ones(geom.vol_shape, device="cuda")
    proj = ConePlan(geom).fp(ones).cpu().numpy().astype(np.float64)
    # analytic chord lengths with numpy (slab method in FP64)
    b = geom.beta.astype(np.float32)
    sb, cb = np.sin(b).astype(np.float64), np.cos(b).astype(np.float64)
    P = geom.P.astype(np.float64)[None, None, :]
    X = geom.xi.astype(np.float64)[None, :, None]
    D = geom.D
    src = [geom.size[0] / 2 - D * sb[:, None, None], geom.size[1] / 2 + D * cb[:, None, None],
           np.full((1, 1, 1), geom.size[2] / 2)]
    d = [P * cb[:, None, None] + D * sb[:, None, None], P * sb[:, None, None] - D * cb[:, None, None],
         X + 0 * P]
    a_in = np.full(proj.shape, -np.inf)
    a_out = np.full(proj.shape, np.inf)
    for a in range(3):
        with np.errstate(divide="ignore", invalid="ignore"):
            t0 = (0 - src[a]) / d[a]
            t1 = (geom.size[a] - src[a]) / d[a]
        a_in = np.maximum(a_in, np.minimum(t0, t1))
        a_out = np.minimum(a_out, np.maximum(t0, t1))
    L = np.clip(a_out - a_in, 0, None) * np.sqrt(d[0] ** 2 + d[1] ** 2 + d[2] ** 2)
    assert rel_l2(proj, L) <= 1e-6


def test_bp_is_linear(torch_cuda):
    from ctgb.device import ConePlan
    torch = torch_cuda
    geom, vol = _random_cone(5)
    plan = ConePlan(geom)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand(geom.sino_shape, device="cuda", generator=g)
    y = torch.rand(geom.sino_shape, device="cuda", generator=g)
    lhs = plan.bp(2.5 * x + y)
    rhs = 2.5 * plan.bp(x) + plan.bp(y)
    assert rel_l2(lhs.cpu().numpy(), rhs.cpu().numpy()) <= 1e-6


def test_fp_residual_fused_matches_unfused(torch_cuda):
    from ctgb.device import ConePlan
    torch = torch_cuda
    geom, vol = _random_cone(9)
    plan = ConePlan(geom)
    x = torch.from_numpy(vol).cuda()
    b = plan.fp(x) * 1.01 + 0.001
    rowsum = plan.fp(torch.ones_like(x))
    out, norms = plan.fp_residual(x, b, rowsum, 1e-6)
    ref = (b - plan.fp(x)) / (rowsum + 1e-6)
    assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) <= 1e-6
    r = (b - plan.fp(x)).double()
    assert abs(norms[0].item() - (r * r).sum().item()) <= 1e-6 * (r * r).sum().item()
    # the norms sum FP32 squares in FP32 warp partials (32 terms), then in FP64
    assert abs(norms[1].item() - (b.double() ** 2).sum().item()) <= 1e-6 * (b.double() ** 2).sum().item()


def test_bp_update_fused_matches_unfused(torch_cuda):
    from ctgb.device import ConePlan
    torch = torch_cuda
    geom, vol = _random_cone(11)
    plan = ConePlan(geom)
    e = torch.rand(geom.sino_shape, device="cuda")
    colsum = plan.bp(torch.ones(geom.sino_shape, device="cuda"))
    x0 = torch.from_numpy(vol).cuda()
    ref = torch.clamp(x0 + 0.7 * plan.bp(e) / (colsum + 1e-3), 0.0, 1.0)
    x = x0.clone()
    plan.bp_update(e, colsum, x, lam=0.7, eps=1e-3, lo=0.0, hi=1.0)
    assert rel_l2(x.cpu().numpy(), ref.cpu().numpy()) <= 1e-6


def test_bad_arguments_raise():
    from ctgb import ops
    from ctgb._lib import CTError
    with pytest.raises(CTError):
        # source inside the volume
        ops.ProjectionCone_3D(np.zeros(8 ** 3, np.float32), 8, 8, 8, [10, 10, 10], [0.1, 0.2], [-1, 0, 1],
                              [-1, 1], 5.0)
    out = ops.ProjectionCone_3D(np.zeros(8 ** 3, np.float32), 8, 8, 8, [10, 10, 10], [0.1, 0.2], [-1, 0, 1],
                                [-1, 1], 5.0, on_error="zeros")
    assert out.shape == (12,) and not out.any()


def test_bp_view_chunks_match_one_pass(oracle, torch_cuda):
    """Backprojection in chunks of views: chunk sums are added in float, so the
    result differs from one pass only by rounding."""
    from ctgb.device import ConePlan
    torch = torch_cuda
    geom, vol = _random_cone(13, nb=30)
    R = torch.rand(geom.sino_shape, device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    one = ConePlan(geom).set_bp_chunk(len(geom.beta))    # one pass
    many = ConePlan(geom).set_bp_chunk(7)                # 5 chunks, the last one shorter
    assert one.bp_chunk_views() == 30 and many.bp_chunk_views() == 7
    a, b = one.bp(R), many.bp(R)
    assert rel_l2(b.cpu().numpy(), a.cpu().numpy()) <= 1e-6
    ref = oracle.cone_bp(R.cpu().numpy(), geom.beta, geom.P, geom.xi, geom.size, geom.D, geom.vol_shape)
    assert rel_l2(b.cpu().numpy(), ref) <= TOL
    colsum = one.bp(torch.ones_like(R))
    x0 = torch.from_numpy(vol).cuda()
    x1, x2 = x0.clone(), x0.clone()
    one.bp_update(R, colsum, x1, lam=0.7, eps=1e-3, lo=0.0, hi=1.0)
    many.bp_update(R, colsum, x2, lam=0.7, eps=1e-3, lo=0.0, hi=1.0)
    assert rel_l2(x2.cpu().numpy(), x1.cpu().numpy()) <= 1e-6
    f1, f2 = one.fdk(R), many.fdk(R)
    assert rel_l2(f2.cpu().numpy(), f1.cpu().numpy()) <= 1e-6


def test_dropin_pinned_overlap_matches_pageable(torch_cuda):
    """Pinned host buffers take the overlapped drop-in path (view chunks copied
    out while the next chunk is projected, copied in while the previous one is
    backprojected; the last chunk runs in z slabs, each copied out while the
    next is summed: 80 slices make three slabs).  The forward projection is the
    same arithmetic per ray, so bit-identical to the pageable path; the
    backprojection adds chunk sums in float, so it differs from one pass only
    by rounding."""
    import ctypes as C
    from ctgb import _lib
    torch = torch_cuda
    geom, vol = _random_cone(17, shape=(80, 28, 32), nb=200, np_=40, nx=24)
    lib = _lib.lib()
    res = np.array([geom.size[0] / geom.nt, geom.size[1] / geom.ns, geom.size[2] / geom.nz])
    size = np.array(geom.size, dtype=np.float64)
    vp = lambda a: C.c_void_p(a.ctypes.data) if isinstance(a, np.ndarray) else C.c_void_p(a.data_ptr())

    def run(h_vol, h_proj, h_back):
        _lib.check(lib.ct_ProjectionCone_3D(vp(h_vol), vp(h_proj), vp(geom.beta), vp(geom.P), vp(geom.xi),
                                            geom.nt, geom.ns, geom.nz, size[0] / 2, size[1] / 2, size[2] / 2,
                                            len(geom.beta), len(geom.P), len(geom.xi), geom.D, vp(res)),
                   "ct_ProjectionCone_3D")
        _lib.check(lib.ct_BackPro(vp(h_back), vp(h_proj), vp(geom.xi), vp(geom.P), vp(geom.beta), geom.D,
                                  len(geom.beta), len(geom.P), len(geom.xi), vp(size), geom.nt, geom.ns, geom.nz),
                   "ct_BackPro")

    page = [np.ascontiguousarray(vol, np.float32), np.zeros(geom.sino_shape, np.float32),
            np.zeros(geom.vol_shape, np.float32)]
    run(*page)
    pin = [torch.empty(s, dtype=torch.float32, pin_memory=True) for s in (geom.vol_shape, geom.sino_shape,
                                                                         geom.vol_shape)]
    pin[0].copy_(torch.from_numpy(page[0]))
    for rep in range(2):                           # the second call reuses the streams and events
        pin[1].fill_(-1.0)
        pin[2].fill_(-1.0)
        run(*pin)
        assert np.array_equal(pin[1].numpy(), page[1])
        assert rel_l2(pin[2].numpy(), page[2]) <= 1e-6
    _lib.check(lib.ct_dropin_release(), "ct_dropin_release")


def test_bp_automatic_chunk():
    """Automatic view chunks: about 768 MiB of packed quads per chunk, evened
    out over the scan (120 views of 768 x 512 at 360 views); small scans in one
    pass."""
    from ctgb.device import ConePlan
    from ctgb.geometry import config_cone_512
    geom = config_cone_512()
    assert ConePlan(geom).bp_chunk_views() == 120
    assert ConePlan(geom.with_views(36)).bp_chunk_views() == 36
    geom_s, _ = _random_cone(5, nb=30)
    assert ConePlan(geom_s).bp_chunk_views() == 30
    assert ConePlan(geom).set_bp_chunk(1000).bp_chunk_views() == 360
