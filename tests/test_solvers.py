"""Reconstruction algorithms of the reference on the device-resident operators
(ctgb/solvers.py): ART on the exported system matrix, cg.m, the TV-CG split
Bregman loop, and the Hessian-Schatten TV loop.

CPU tests check the algebraic pieces against their MATLAB definitions and
properties (an explicit Kaczmarz sweep, a dense solve, Sobel responses, the
adjointness of the Hessian operator pair); GPU tests run the loops through
the projectors.
"""
import math

import numpy as np
import pytest
import torch

from conftest import rel_l2


def test_cg_solves_spd_system():
    from ctgb.solvers import cg
    rng = np.random.default_rng(0)
    M = rng.standard_normal((40, 40))
    A = torch.from_numpy(M @ M.T + 40 * np.eye(40))
    b = torch.from_numpy(rng.standard_normal(40))
    res = cg(lambda v: A @ v, b, tol=1e-12, maxit=200)
    assert res.flag == 1 and res.iterations < 200
    np.testing.assert_allclose(res.x.numpy(), np.linalg.solve(A.numpy(), b.numpy()), rtol=1e-8, atol=1e-10)
    # cg.m's stopping rule is relative to the starting residual: a warm start
    # near the solution still reaches the same solution
    x0 = res.x + 1e-3 * torch.from_numpy(rng.standard_normal(40))
    np.testing.assert_allclose(cg(lambda v: A @ v, b, tol=1e-10, maxit=200, x0=x0).x.numpy(), res.x.numpy(),
                               rtol=1e-7, atol=1e-10)


def test_gradient_matrices_follow_gradient2dmatrix():
    from ctgb.solvers import gradient2d_matrices
    n = 9
    gx, gy = gradient2d_matrices(n, n)
    yy, xx = np.mgrid[0:n, 0:n].astype(np.float64)
    ramp_x = (2.0 * xx + 0.5 * yy).ravel()          # pixel (y, x), x fastest
    gxr = (gx @ ramp_x).reshape(n, n)
    gyr = (gy @ ramp_x).reshape(n, n)
    # Sobel: 4 x (2 * slope) in the interior; one-sided at the mirrored edges
    np.testing.assert_allclose(gxr[1:-1, 1:-1], 4 * 2 * 2.0)
    np.testing.assert_allclose(gyr[1:-1, 1:-1], 4 * 2 * 0.5)
    np.testing.assert_allclose(gxr[1:-1, 0], 4 * 2.0)
    assert abs(gx @ np.ones(n * n)).max() == 0 and abs(gy @ np.ones(n * n)).max() == 0


def test_soft_threshold_and_cut():
    from ctgb.solvers import cut, soft_threshold
    x = torch.tensor([-3.0, -1.0, -0.5, 0.0, 0.5, 1.0, 3.0])
    np.testing.assert_allclose(soft_threshold(x, 1.0).numpy(), [-2, 0, 0, 0, 0, 0, 2])
    np.testing.assert_allclose(cut(x, 1.0).numpy(), [-1, 0, -0.5, 0, 0.5, 0, 1])    # +-t itself maps to 0


def test_hessian_operator_pair_is_adjoint():
    from ctgb.solvers import hessian_log3d, hessian_log_templates, hstar_omega
    H = hessian_log_templates(3).double()
    assert torch.allclose(H, H.transpose(0, 1))                          # symmetric Hessian templates
    g = torch.Generator().manual_seed(1)
    u = torch.rand((7, 8, 9), generator=g, dtype=torch.float64)
    om = torch.rand((3, 3, 7, 8, 9), generator=g, dtype=torch.float64)
    lhs = float((hessian_log3d(u, H) * om).sum())
    rhs = float((u * hstar_omega(om, H)).sum())
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    # each component is MATLAB's convn(u, H_ij, 'same') (scipy's 'same' convolution)
    from scipy.signal import convolve
    hs = hessian_log3d(u, H)
    for i, j in [(0, 0), (0, 1), (2, 1)]:
        np.testing.assert_allclose(hs[i, j].numpy(), convolve(u.numpy(), H[i, j].numpy(), mode="same"),
                                   rtol=1e-12, atol=1e-15)
    # the templates as HessianLOGtemplate3D.m writes them (coordinates i - (ps - 1)/2, i = 1..ps)
    e = math.exp(-(1 + 4 + 0) / 2)
    assert float(H[0, 1, 1, 2, 0]) == pytest.approx(1 * 2 * e / (2 * math.pi) ** 3, rel=1e-14)


@pytest.mark.gpu
def test_art_matches_explicit_kaczmarz_and_converges():
    from ctgb import phantom
    from ctgb.device import ParPlan
    from ctgb.solvers import art
    n = 32
    theta = np.arange(1, 61) * np.pi / 60
    T = np.linspace(-24.5, 24.5, 50)
    plan = ParPlan(n, n, (1.0, 1.0), theta, T)
    img = phantom.ellipses_2d(n, n, phantom.ellipse_params(6, seed=2), device="cuda")
    A = plan.sysmat()
    b = plan.fp(img).reshape(-1)
    # one sweep against the MATLAB loop (ART.m:57-75) on the same rows, in float64
    As = A.to_scipy().astype(np.float64)
    bn = b.cpu().numpy().astype(np.float64)
    x = np.zeros(n * n)
    for j in range(As.shape[0]):
        lo, hi = As.indptr[j], As.indptr[j + 1]
        cols, vals = As.indices[lo:hi], As.data[lo:hi]
        nn = vals @ vals
        if nn != 0:
            x[cols] -= 0.3 * vals * (vals @ x[cols] - bn[j]) / nn
    x1 = art(A, b, lam=0.3, sweeps=1).cpu().numpy()
    assert rel_l2(x1, x) <= 1e-4
    err = [rel_l2(art(A, b, lam=0.3, sweeps=k).cpu().numpy(), img.cpu().numpy().ravel()) for k in (1, 4, 16)]
    assert err[0] > err[1] > err[2] and err[2] < 0.1


@pytest.mark.gpu
def test_tv_cg_reconstructs_fan_scan():
    from ctgb import phantom
    from ctgb.device import FanPlan
    from ctgb.geometry import fan_config
    from ctgb.solvers import tv_cg
    n = 32
    g = fan_config(n, 72, 64, 90.0, float(n))
    plan = FanPlan(g)
    img = phantom.ellipses_2d(n, n, phantom.ellipse_params(6, seed=5), device="cuda")
    R = plan.fp(img).reshape(-1)
    A = plan.sysmat()
    res = tv_cg(A, R, n, n, mu=200.0, lam=0.2, iter_cg=40, outer=2, inner=3)
    e = rel_l2(res.x.float().cpu().numpy(), img.cpu().numpy().ravel())
    assert e < 0.1
    assert res.loss[-1] <= res.loss[0]


@pytest.mark.gpu
def test_hessian_schatten_tv_decreases_objective():
    from ctgb import phantom
    from ctgb.device import ConePlan
    from ctgb.geometry import ConeGeometry, centred_domain, view_angles
    from ctgb.solvers import hessian_schatten_tv
    n = 16
    geom = ConeGeometry(n, n, n, (16.0, 16.0, 16.0), view_angles(36), centred_domain(33, 0.75),
                        centred_domain(33, 0.75), 60.0)
    plan = ConePlan(geom)
    vol = phantom.ellipsoids_3d(n, n, n, phantom.ellipsoid_params(5, seed=6), device="cuda")
    V = plan.fp(vol)
    u0 = plan.fdk(V).double()
    res = hessian_schatten_tv(plan, V, u0, alpha=2e3, tau=1e-3, outer=3, inner=3)
    obj = res.objective
    assert res.outer_iterations >= 1
    assert all(b <= a * (1 + 1e-12) for a, b in zip(obj, obj[1:]))      # monotone choice of U
    assert obj[-1] < obj[0]
