"""SIRT / SIRT3D / SIRT-TV loops: host logic on CPU, parity with the oracle on GPU."""
import numpy as np
import pytest
import torch

from conftest import rel_l2


# ---------------------------------------------------------------------------
# CPU: the driver logic with a dense-matrix stand-in for the operators
# ---------------------------------------------------------------------------
class DensePlan:
    """fp/bp/fp_residual/bp_update over explicit matrices (CPU tensors)."""

    def __init__(self, A, B, shape):
        self.A, self.B = A, B

        class G:
            img_shape = shape
        self.geom = G()

    def fp(self, x, out=None):
        return (self.A @ x.reshape(-1).double()).float()

    def bp(self, y, out=None):
        return (self.B @ y.reshape(-1).double()).float().reshape(self.geom.img_shape)

    def fp_residual(self, x, b, rowsum=None, eps=0.0, out=None, norms=None):
        r = (b.double() - self.A @ x.reshape(-1).double())
        sc = 1.0 / (rowsum.double() + eps) if rowsum is not None else 1.0
        out.copy_((r * sc).float())
        norms[0] += float((r * r).sum())
        norms[1] += float((b.double() ** 2).sum())
        return out, norms

    def bp_update(self, e, colsum, x, lam=1.0, eps=0.0, lo=0.0, hi=float("inf")):
        upd = (self.B @ e.double()).reshape(x.shape) / (colsum.double() + eps)
        x.copy_(torch.clamp(x.double() + lam * upd, lo, hi).float())
        return x


def _dense_problem(seed=0, n=12, m=40):
    rng = np.random.default_rng(seed)
    A = torch.from_numpy(rng.uniform(0, 1, (m, n * n)))
    B = A.T.clone()
    x_true = torch.from_numpy(rng.uniform(0, 1, (n, n))).float()
    b = (A @ x_true.reshape(-1).double()).float()
    return DensePlan(A, B, (n, n)), b, x_true


def test_sirt_driver_matches_explicit_loop():
    from ctgb.sirt import Sirt, SirtConfig
    from oracle.oracle import sirt_loop
    plan, b, _ = _dense_problem()
    cfg = SirtConfig(iters=7, lam=1.5, lo=0.0, hi=1.0, eps=1e-9)
    res = Sirt(plan, b, cfg).run()
    A = plan.A.numpy()
    ref = sirt_loop(lambda x: A @ x.ravel(), lambda y: (A.T @ y).reshape(12, 12), b.numpy(), np.zeros((12, 12)),
                    7, 1.5, 0.0, 1.0, 1e-9)
    assert res.iterations == 7
    assert rel_l2(res.x.numpy(), ref) <= 1e-5
    # residual history is non-increasing for this well-posed problem
    r = [v for _, v in res.residuals]
    assert all(r[i + 1] <= r[i] * (1 + 1e-6) for i in range(len(r) - 1))


def test_sirt_tolerance_stops_early():
    from ctgb.sirt import Sirt, SirtConfig
    plan, b, _ = _dense_problem(1)
    full = Sirt(plan, b, SirtConfig(iters=200, lam=1.0, eps=1e-9)).run()
    target = full.residuals[20][1]
    res = Sirt(plan, b, SirtConfig(iters=200, lam=1.0, eps=1e-9, tol=target)).run()
    assert res.iterations <= 22 and res.residuals[-1][1] <= target


def test_sirt_checkpoint_resume_is_exact(tmp_path):
    from ctgb.sirt import Sirt, SirtConfig, load_checkpoint
    plan, b, _ = _dense_problem(2)
    ck = tmp_path / "state.npz"
    straight = Sirt(plan, b, SirtConfig(iters=8, lam=1.0)).run()
    Sirt(plan, b, SirtConfig(iters=4, lam=1.0, checkpoint=str(ck), checkpoint_every=4)).run()
    x, it, hist = load_checkpoint(ck, device="cpu")
    assert it == 4 and len(hist) == 4
    resumed = Sirt(plan, b, SirtConfig(iters=8, lam=1.0)).run(x0=x, start_iter=it, residuals=hist)
    assert resumed.iterations == 8
    assert torch.equal(resumed.x, straight.x)
    assert [r for _, r in resumed.residuals] == [r for _, r in straight.residuals]


def test_tv_oracle_properties():
    from oracle.oracle import tv_flow
    rng = np.random.default_rng(3)
    const = np.full((6, 7, 8), 0.3)
    assert np.allclose(tv_flow(const, 5, 1e-2), const)          # a constant has zero TV gradient
    x = np.clip(0.5 + 0.2 * rng.normal(size=(8, 9, 10)), 0, None)

    def tv(v):
        dx = np.diff(v, axis=2, append=v[:, :, -1:])
        dy = np.diff(v, axis=1, append=v[:, -1:, :])
        dz = np.diff(v, axis=0, append=v[-1:, :, :])
        return np.sqrt(dx * dx + dy * dy + dz * dz + 1e-16).sum()
    y = tv_flow(x, 10, 1e-3)
    assert tv(y) < tv(x)
    assert y.min() >= 0.0
    step_rms = np.sqrt(np.mean((tv_flow(x, 1, 1e-3, lo=-1e9) - x) ** 2))
    assert abs(step_rms - 1e-3) < 1e-9                          # normalised: each sub-step moves RMS `step`


def test_metrics_match_reference_formulas():
    from ctgb.sirt import rrmse, local_error, psnr
    rng = np.random.default_rng(4)
    a, b = rng.random(50), rng.random(50)
    assert abs(rrmse(a, b) - np.sqrt(np.mean((a - b) ** 2)) / (np.sqrt(np.mean(b ** 2)) + 2.220446049250313e-16)) < 1e-15
    assert abs(local_error(a, b) - np.linalg.norm(a - b) / np.linalg.norm(b)) < 1e-15
    assert psnr(b, b) == float("inf")


# ---------------------------------------------------------------------------
# GPU: the fused device loop against the oracle loop
# ---------------------------------------------------------------------------
def _small_cone(seed=5):
    from ctgb.geometry import ConeGeometry, view_angles, centred_domain
    from ctgb import phantom
    geom = ConeGeometry(24, 24, 20, (24.0, 24.0, 20.0), view_angles(30), centred_domain(48, 0.8),
                        centred_domain(40, 0.7), 70.0)
    vol = phantom.ellipsoids_3d(24, 24, 20, phantom.ellipsoid_params(8, seed=seed)).numpy()
    return geom, vol


@pytest.mark.gpu
def test_sirt3d_matches_oracle_loop(oracle):
    from ctgb.device import ConePlan
    from ctgb.sirt import Sirt, SirtConfig
    from oracle.oracle import sirt_loop
    geom, vol = _small_cone()
    b = oracle.cone_fp(vol, geom.beta, geom.P, geom.xi, geom.size, geom.D)
    plan = ConePlan(geom)
    res = Sirt(plan, torch.from_numpy(b).cuda(), SirtConfig(iters=4, lam=1.0, eps=1e-9)).run()
    fp = lambda x: oracle.cone_fp(x.astype(np.float32), geom.beta, geom.P, geom.xi, geom.size, geom.D)
    bp = lambda y: oracle.cone_bp(y.astype(np.float32), geom.beta, geom.P, geom.xi, geom.size, geom.D, geom.vol_shape)
    ref = sirt_loop(fp, bp, b, np.zeros(geom.vol_shape), 4, 1.0, 0.0, np.inf, 1e-9)
    assert rel_l2(res.x.cpu().numpy(), ref) <= 1e-4
    r = [v for _, v in res.residuals]
    assert r[-1] < r[0]


@pytest.mark.gpu
def test_tv_flow_matches_oracle():
    from ctgb.device import tv_flow
    from oracle.oracle import tv_flow as tv_ref
    rng = np.random.default_rng(6)
    x = np.clip(0.5 + 0.2 * rng.normal(size=(10, 12, 14)), 0, None).astype(np.float32)
    out = tv_flow(torch.from_numpy(x).cuda(), 5, 1e-3, 1e-8, 0.0).cpu().numpy()
    ref = tv_ref(x, 5, 1e-3, 1e-8, 0.0)
    assert rel_l2(out - x, ref - x) <= 1e-4          # the change itself, not just the image
    img = x[3]
    out2 = tv_flow(torch.from_numpy(img.copy()).cuda(), 3, 1e-3).cpu().numpy()
    assert rel_l2(out2 - img, tv_ref(img, 3, 1e-3) - img) <= 1e-4
    # a volume with more z blocks than the launch holds: threads walk z with the grid's stride
    big = np.clip(0.5 + 0.2 * rng.normal(size=(128, 160, 96)), 0, None).astype(np.float32)
    out3 = tv_flow(torch.from_numpy(big).cuda(), 2, 1e-3, 1e-8, 0.0).cpu().numpy()
    assert rel_l2(out3 - big, tv_ref(big, 2, 1e-3, 1e-8, 0.0) - big) <= 1e-4


@pytest.mark.gpu
def test_sirt_tv_graph_replay_equals_eager():
    from ctgb.device import ConePlan
    from ctgb.sirt import Sirt, SirtConfig
    geom, vol = _small_cone(7)
    plan = ConePlan(geom)
    b = plan.fp(torch.from_numpy(vol).cuda())
    cfg = dict(iters=5, lam=1.0, eps=1e-9, tv_iters=4, tv_step=1e-3)
    eager = Sirt(plan, b, SirtConfig(**cfg)).run()
    graph = Sirt(plan, b, SirtConfig(use_graph=True, **cfg)).run()
    assert torch.equal(eager.x, graph.x)            # the image kernels are deterministic
    # the residual norms are double atomics: summation order may differ in the last bit
    for (i0, r0), (i1, r1) in zip(eager.residuals, graph.residuals):
        assert i0 == i1 and abs(r0 - r1) <= 1e-12 * abs(r0)


@pytest.mark.gpu
def test_fan_sirt_matches_oracle_loop(oracle):
    from ctgb.device import FanPlan
    from ctgb.geometry import fan_config
    from ctgb.sirt import Sirt, SirtConfig, MATLAB_EPS
    from ctgb import phantom
    from oracle.oracle import sirt_loop
    geom = fan_config(40, 36, 64, 120.0, 40.0)
    img = phantom.ellipses_2d(40, 40, phantom.ellipse_params(10, seed=8)).numpy()
    b = oracle.fan_fp(img, geom.beta, geom.P, geom.size, geom.D).astype(np.float32)
    plan = FanPlan(geom)
    res = Sirt(plan, torch.from_numpy(b).cuda(), SirtConfig(iters=5, lam=2.0, lo=0.0, hi=1.0, eps=MATLAB_EPS)).run()
    fp = lambda x: oracle.fan_fp(x.astype(np.float32), geom.beta, geom.P, geom.size, geom.D)
    bp = lambda y: oracle.fan_bp(y.astype(np.float32), geom.beta.astype(np.float32), geom.P.astype(np.float32),
                                 geom.size, geom.img_shape, geom.D)
    ref = sirt_loop(fp, bp, b, np.zeros(geom.img_shape), 5, 2.0, 0.0, 1.0, MATLAB_EPS)
    assert rel_l2(res.x.cpu().numpy(), ref) <= 1e-4
