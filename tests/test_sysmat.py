"""System-matrix export (ct_fan_sysmat, ct_cone_sysmat) on the GPU.

The CSR rows come from the projectors' own walks, so A x must equal the
forward projection to float rounding; the 2D matrices must also equal the
reference's MATLAB builders (GenSysMatFan.m / GenSysMatParal.m, restated in
oracle/sysmat.py) entry by entry.
"""
import math

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_fan_sysmat_equals_gensysmatfan():
    import torch
    from ctgb.device import FanPlan
    from ctgb.geometry import FanGeometry
    from oracle.sysmat import gensysmat_fan
    n, D = 24, 60.0
    beta = np.arange(1, 13) * 2 * np.pi / 12 + 0.013
    P = np.linspace(-17.3, 17.3, 31)
    plan = FanPlan(FanGeometry(n, n, (24.0, 24.0), beta, P, D))
    A = plan.sysmat().to_scipy()
    ref = gensysmat_fan(n, n, [24.0, 24.0], beta, P, D, 12.0, 12.0)
    assert A.shape == ref.shape
    d = A.astype(np.float64) - ref
    assert abs(d).max() <= 1e-5                        # every entry, in mm
    assert rel_l2(A.toarray(), ref.toarray()) <= 1e-6
    # same pattern: no entry above 1e-6 mm on one side only
    big = lambda m: {(r, c) for r, c, v in zip(*m.nonzero(), m[m.nonzero()].A1) if v > 1e-6}
    assert big(A) == big(ref)


def test_parallel_sysmat_equals_gensysmatparal(oracle):
    """The reference's parallel-beam matrix builder (GenSysMatParal.m) and its
    projector (ProjectionParallel_2D.cu) disagree on some rays (the projector
    drops some lines through the image and snaps crossings within 1e-5 of a
    grid line); the export follows the projector.  On the rays where the two
    references agree, the export equals the MATLAB matrix."""
    from ctgb.device import ParPlan
    from oracle.sysmat import gensysmat_paral
    n = 24
    theta = np.arange(12) * np.pi / 12 + 0.0137
    T = np.linspace(-18.3, 18.3, 37)
    plan = ParPlan(n, n, (1.0, 1.0), theta, T)
    A = plan.sysmat().to_scipy().astype(np.float64)
    ref = gensysmat_paral(n, n, [24.0, 24.0], 12.0, 12.0, theta, T)
    assert A.shape == ref.shape
    img = np.random.default_rng(0).random((n, n)).astype(np.float32)
    proj = oracle.par_fp(img, theta, T, np.array([24.0, 24.0])).ravel()
    agree = np.abs(ref @ img.ravel().astype(np.float64) - proj) <= 1e-6 * np.abs(proj).max()
    assert agree.mean() > 0.9
    rows = np.flatnonzero(agree)
    assert rel_l2(A[rows].toarray(), ref[rows].toarray()) <= 1e-6


def test_parallel_sysmat_times_image_is_the_projection():
    """Including lines whose end points lie inside the image (max t 16.5 below
    the half diagonal 16.97): the export follows the projector there."""
    import torch
    from ctgb.device import ParPlan
    n = 24
    theta = np.arange(12) * np.pi / 12 + 0.01
    T = np.linspace(-16.5, 16.5, 34)
    plan = ParPlan(n, n, (1.0, 1.0), theta, T)
    img = torch.rand((n, n), generator=torch.Generator().manual_seed(0)).cuda()
    ax = plan.sysmat().matvec(img).view(len(theta), len(T))
    assert rel_l2(ax.cpu().numpy(), plan.fp(img).cpu().numpy()) <= 1e-6


@pytest.mark.parametrize("grazing", [False, True])
def test_fan_sysmat_times_image_is_the_projection(grazing):
    import torch
    from ctgb import phantom
    from ctgb.device import FanPlan
    from ctgb.geometry import FanGeometry
    n = 40
    if grazing:      # bin at P = 0 and views at multiples of pi/2: rays along grid lines
        beta = np.arange(8) * np.pi / 2 / 2
        P = np.linspace(-30, 30, 41)
    else:
        beta = np.arange(1, 31) * 2 * np.pi / 30
        P = np.linspace(-31.0, 31.0, 57)
    plan = FanPlan(FanGeometry(n, n, (40.0, 40.0), beta, P, 90.0))
    img = phantom.ellipses_2d(n, n, phantom.ellipse_params(8, seed=3), device="cuda")
    A = plan.sysmat()
    ax = A.matvec(img).view(len(beta), len(P))
    fp = plan.fp(img)
    assert rel_l2(ax.cpu().numpy(), fp.cpu().numpy()) <= 1e-6
    assert A.nnz > 0 and int(A.row_ptr[-1]) == A.nnz


def test_cone_sysmat_times_volume_is_the_projection():
    import torch
    from ctgb import phantom
    from ctgb.device import ConePlan
    from ctgb.geometry import ConeGeometry, centred_domain, view_angles
    nz, ns, nt = 14, 18, 20
    geom = ConeGeometry(nt, ns, nz, (10.0, 9.0, 7.0), view_angles(12), centred_domain(27, 0.45),
                        centred_domain(21, 0.42), 40.0)
    vol = phantom.ellipsoids_3d(nt, ns, nz, phantom.ellipsoid_params(8, seed=4), device="cuda")
    plan = ConePlan(geom)
    fp = plan.fp(vol)
    A = plan.sysmat()
    assert rel_l2(A.matvec(vol).view(fp.shape).cpu().numpy(), fp.cpu().numpy()) <= 1e-6
    # a view range gives the matching block of rows
    B = plan.sysmat(view0=5, nviews=3)
    assert B.shape == (3 * 21 * 27, nt * ns * nz)
    assert rel_l2(B.matvec(vol).view(3, 21, 27).cpu().numpy(), fp[5:8].cpu().numpy()) <= 1e-6


def test_cone_sysmat_grazing_rays():
    """Views at multiples of pi/2 with bins and rows through the centre: rays
    along grid planes take the FP64 reference walk in both the projector and
    the export."""
    import torch
    from ctgb import phantom
    from ctgb.device import ConePlan
    from ctgb.geometry import ConeGeometry
    nz, ns, nt = 10, 12, 12
    beta = (np.arange(4) * np.pi / 2).astype(np.float32)
    P = ((np.arange(19) - 9) * 0.8).astype(np.float32)
    xi = ((np.arange(13) - 6) * 0.7).astype(np.float32)
    geom = ConeGeometry(nt, ns, nz, (12.0, 12.0, 10.0), beta, P, xi, 40.0)
    vol = phantom.ellipsoids_3d(nt, ns, nz, phantom.ellipsoid_params(6, seed=9), device="cuda")
    plan = ConePlan(geom)
    fp = plan.fp(vol)
    A = plan.sysmat()
    assert rel_l2(A.matvec(vol).view(fp.shape).cpu().numpy(), fp.cpu().numpy()) <= 1e-6


def test_sysmat_rejects_short_arrays():
    import ctypes as C
    import torch
    from ctgb import _lib
    from ctgb.device import FanPlan
    from ctgb.geometry import FanGeometry
    plan = FanPlan(FanGeometry(16, 16, (16.0, 16.0), np.arange(6) * 0.5, np.linspace(-12, 12, 20), 40.0))
    rp = torch.empty(6 * 20 + 1, dtype=torch.int64, device="cuda")
    col = torch.empty(4, dtype=torch.int32, device="cuda")
    val = torch.empty(4, dtype=torch.float32, device="cuda")
    nnz = C.c_longlong()
    st = _lib.lib().ct_fan_sysmat(plan._h, C.c_void_p(rp.data_ptr()), C.c_void_p(col.data_ptr()),
                                  C.c_void_p(val.data_ptr()), 4, C.byref(nnz), None)
    assert st == 1 and nnz.value > 4
