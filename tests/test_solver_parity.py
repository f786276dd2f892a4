"""The TV-CG and Hessian-Schatten TV callers against FP64 restatements of the
reference's MATLAB loops (oracle/solvers.py: TVCG.m:58-142 with cg.m,
soft_threshold.m, Cut.m, LocalError.m, gradient2Dmatrix_x/y.m;
HessianSchattenTV.m:66-175 with its helper files).

CPU: ctgb.solvers run on CPU tensors with the same operators as the
restatement (the oracle's system matrix / projectors), so the comparison pins
the loop logic itself (float64 both sides: rel-L2 <= 1e-9).
GPU: ctgb.solvers with the GPU operators (exported CSR matrix, cone plan)
against the restatement with the oracle's operators (GenSysMatFan.m restated;
the reference kernels restated): rel-L2 <= 1e-4 after a few iterations
(operator differences ~1e-7 amplified by CG / the Nesterov loop).
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2


def _fan_case(n=20, views=30, bins=40, seed=5):
    from ctgb import phantom
    from ctgb.geometry import fan_config
    from oracle.sysmat import gensysmat_fan
    g = fan_config(n, views, bins, 80.0, float(n))
    img = phantom.ellipses_2d(n, n, phantom.ellipse_params(6, seed=seed)).numpy().astype(np.float64)
    A = gensysmat_fan(n, n, g.size, g.beta, g.P, g.D, g.size[0] / 2, g.size[1] / 2)
    return g, img, A


def _csr_from_scipy(A, device):
    from ctgb.device import CsrMatrix
    A = A.tocsr()
    return CsrMatrix(torch.from_numpy(A.indptr.astype(np.int64)).to(device),
                     torch.from_numpy(A.indices.astype(np.int32)).to(device),
                     torch.from_numpy(A.data.astype(np.float32)).to(device), A.shape)


TVCG_ARGS = dict(mu=200.0, lam=0.2, iter_cg=25, outer=2, inner=3)


def test_tvcg_loop_matches_restatement_cpu():
    from ctgb.solvers import tv_cg
    from oracle.solvers import tvcg
    g, img, A = _fan_case()
    A32 = A.astype(np.float32).astype(np.float64)          # the values the CSR export carries
    R = A32 @ img.ravel()
    n = g.nt
    ref, ref_loss = tvcg(A32, R, n, n, miu=200.0, lamda1=0.2, iter_cg=25, outeriter=2, inner=3)
    res = tv_cg(_csr_from_scipy(A, "cpu"), torch.from_numpy(R), n, n, **TVCG_ARGS)
    assert rel_l2(res.x.numpy(), ref) <= 1e-9
    assert len(res.loss) == len(ref_loss)
    np.testing.assert_allclose(res.loss, ref_loss, rtol=1e-7)


@pytest.mark.gpu
def test_tvcg_on_gpu_export_matches_restatement():
    from ctgb.device import FanPlan
    from ctgb.solvers import tv_cg
    from oracle.solvers import tvcg
    g, img, A = _fan_case()
    n = g.nt
    R = A @ img.ravel()
    ref, _ = tvcg(A, R, n, n, miu=200.0, lamda1=0.2, iter_cg=25, outeriter=2, inner=3)
    res = tv_cg(FanPlan(g).sysmat(), torch.from_numpy(R).cuda(), n, n, **TVCG_ARGS)
    assert rel_l2(res.x.cpu().numpy(), ref) <= 1e-4


class _OracleCone:
    """Cone operators of the oracle behind the plan interface (CPU tensors)."""

    def __init__(self, geom, oracle):
        self.g, self.o = geom, oracle

    def fp(self, x):
        g = self.g
        return torch.from_numpy(self.o.cone_fp(x.numpy().astype(np.float32), g.beta, g.P, g.xi, g.size, g.D))

    def bp(self, y):
        g = self.g
        return torch.from_numpy(self.o.cone_bp(y.numpy().astype(np.float32), g.beta, g.P, g.xi, g.size, g.D,
                                               g.vol_shape))


def _cone_case(oracle, n=10):
    from ctgb import phantom
    from ctgb.geometry import ConeGeometry, centred_domain, view_angles
    geom = ConeGeometry(n, n, n, (float(n),) * 3, view_angles(24), centred_domain(21, 0.75),
                        centred_domain(21, 0.75), 40.0)
    vol = phantom.ellipsoids_3d(n, n, n, phantom.ellipsoid_params(5, seed=6)).numpy()
    V = oracle.cone_fp(vol, geom.beta, geom.P, geom.xi, geom.size, geom.D).astype(np.float32)
    U0 = oracle.fdk(V, geom.beta, geom.P, geom.xi, geom.size, geom.D, geom.vol_shape).astype(np.float64)
    return geom, V, U0


HST_ARGS = dict(alpha=2e3, tau=1e-3, order=2)


def _hst_reference(oracle, geom, V, U0, outer, inner):
    from oracle.solvers import hessian_schatten_tv as ref_hst
    fp = lambda x: oracle.cone_fp(x, geom.beta, geom.P, geom.xi, geom.size, geom.D).astype(np.float64)
    bp = lambda y: oracle.cone_bp(y, geom.beta, geom.P, geom.xi, geom.size, geom.D, geom.vol_shape).astype(np.float64)
    return ref_hst(fp, bp, V.astype(np.float64), U0, tmm=outer, tnesterov=inner, **HST_ARGS)


def test_hst_loop_matches_restatement_cpu(oracle):
    from ctgb.solvers import hessian_schatten_tv
    geom, V, U0 = _cone_case(oracle)
    ref_u, ref_obj, ref_t = _hst_reference(oracle, geom, V, U0, 2, 3)
    res = hessian_schatten_tv(_OracleCone(geom, oracle), torch.from_numpy(V), torch.from_numpy(U0), outer=2, inner=3,
                              **HST_ARGS)
    assert res.outer_iterations == ref_t
    assert rel_l2(res.x.numpy(), ref_u) <= 1e-9
    np.testing.assert_allclose(res.objective, ref_obj, rtol=1e-7)      # residual rounded to float32 in the product


@pytest.mark.gpu
def test_hst_on_gpu_operators_matches_restatement(oracle):
    from ctgb.device import ConePlan
    from ctgb.solvers import hessian_schatten_tv
    geom, V, U0 = _cone_case(oracle)
    ref_u, ref_obj, ref_t = _hst_reference(oracle, geom, V, U0, 2, 3)
    res = hessian_schatten_tv(ConePlan(geom), torch.from_numpy(V).cuda(), torch.from_numpy(U0).cuda(), outer=2,
                              inner=3, **HST_ARGS)
    assert res.outer_iterations == ref_t
    assert rel_l2(res.x.cpu().numpy(), ref_u) <= 1e-4
    np.testing.assert_allclose(res.objective, ref_obj, rtol=1e-4)
