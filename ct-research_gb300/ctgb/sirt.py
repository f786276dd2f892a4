"""SIRT / SIRT3D / SIRT-TV reconstruction loops on device-resident operators.

The reference iterates (Iterative_algorithm/SIRT.m:121-144, GPU operator form
in the comments at :123-124 and :131; SIRT3D.m:67-92):

    rowsum = A 1,  colsum = A^T 1                      (SIRT.m:123-124)
    x <- clamp(x + lam * A^T((b - A x) / (rowsum + eps)) / (colsum + eps), lo, hi)

with lam = 2, x in [0, 1], eps = MATLAB eps and an FBPfan start for 2D fan
SIRT (SIRT.m:102-113), lam = 1, x >= 0, eps = 1e-9 and a zero start for
SIRT3D.  A is the Siddon forward projector and A^T the voxel-driven
backprojector of the same geometry, so the normalisers come from the same
operators (A^T is not the exact adjoint of A).

Each iteration here is two kernel launches: the forward projection fused with
the residual, its scaling and the residual norms (ct_*_fp_residual), and the
backprojection fused with the update and clamp (ct_*_bp_update).  SIRT-TV adds
`tv_iters` normalised isotropic TV gradient-flow sub-steps after every SIRT
step (the 3D, forward-difference form of the TV flow of tv.m:30-44).

The whole iteration can be captured once into a CUDA graph and replayed.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np
import torch

from . import device as dev

MATLAB_EPS = 2.220446049250313e-16


@dataclass
class SirtConfig:
    iters: int = 50
    lam: float = 1.0             # relaxation (SIRT3D.m:69; SIRT.m:102 uses 2)
    lo: float = 0.0              # clamp range (SIRT.m:104: [0, 1]; SIRT3D.m:82: x >= 0)
    hi: float = float("inf")
    eps: float = 1e-9            # normaliser guard (SIRT3D.m:81; SIRT.m uses MATLAB eps)
    tv_iters: int = 0            # TV sub-iterations per outer iteration (0: plain SIRT)
    tv_step: float = 1e-3        # RMS size of one TV sub-step
    tv_eps: float = 1e-8         # gradient-norm smoothing of TV_eps
    tol: float = 0.0             # stop when ||b - A x|| / ||b|| <= tol
    check_every: int = 1         # iterations between residual checks (host sync)
    use_graph: bool = False      # replay the iteration from a captured CUDA graph
    checkpoint: str | None = None
    checkpoint_every: int = 0
    # Rays whose path through the volume is shorter than min_rowsum (mm) and
    # voxels whose colsum is below min_colsum_frac * max(colsum) take no part
    # in the update.  0 keeps every ray and voxel, as the reference does; with
    # noisy data a corner-clipping ray has a tiny rowsum, and dividing its
    # noise by it drives the unmatched voxel-driven A^T to diverge.
    min_rowsum: float = 0.0
    min_colsum_frac: float = 0.0


@dataclass
class SirtResult:
    x: torch.Tensor
    iterations: int
    residuals: list = field(default_factory=list)   # relative data residual after each checked iteration
    seconds: float = 0.0


def relative_residual(norms: torch.Tensor) -> float:
    n = norms.detach().cpu().numpy()
    return float(math.sqrt(n[0]) / math.sqrt(n[1])) if n[1] > 0 else float("nan")


class Sirt:
    """SIRT(-TV) over a ConePlan or FanPlan (anything with fp/bp/fp_residual/bp_update)."""

    def __init__(self, plan, b: torch.Tensor, cfg: SirtConfig):
        self.plan, self.b, self.cfg = plan, b, cfg
        ones_x = torch.ones(self._x_shape(), dtype=torch.float32, device=b.device)
        ones_b = torch.ones_like(b)
        self.rowsum = plan.fp(ones_x)
        self.colsum = plan.bp(ones_b)
        # an infinite normaliser makes 1 / (sum + eps) exactly 0: the ray / voxel drops out
        if cfg.min_rowsum > 0:
            self.rowsum[self.rowsum < cfg.min_rowsum] = float("inf")
        if cfg.min_colsum_frac > 0:
            self.colsum[self.colsum < cfg.min_colsum_frac * float(self.colsum.max())] = float("inf")
        self.e = torch.empty_like(b)
        self.norms = torch.zeros(2, dtype=torch.float64, device=b.device)
        self.tv_work = torch.empty_like(ones_x) if cfg.tv_iters > 0 else None
        self.tv_scratch = torch.zeros(2, dtype=torch.float64, device=b.device)
        self.tv = getattr(plan, "tv_flow", dev.tv_flow)
        self.graph = None
        self.x = None

    def _x_shape(self):
        g = self.plan.geom
        return g.vol_shape if hasattr(g, "vol_shape") else g.img_shape

    # one iteration: fused residual FP, fused update BP, optional TV flow
    def _step(self, x):
        self.norms.zero_()
        self.plan.fp_residual(x, self.b, self.rowsum, self.cfg.eps, out=self.e, norms=self.norms)
        self.plan.bp_update(self.e, self.colsum, x, lam=self.cfg.lam, eps=self.cfg.eps, lo=self.cfg.lo,
                            hi=self.cfg.hi)
        if self.cfg.tv_iters > 0:
            self.tv(x, self.cfg.tv_iters, self.cfg.tv_step, self.cfg.tv_eps, self.cfg.lo, self.tv_work,
                    self.tv_scratch)

    def _capture(self, x):
        # warm-up: the first call allocates plan workspaces (not allowed in capture)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            tmp = x.clone()
            self._step(tmp)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._step(x)
        return g

    def run(self, x0: torch.Tensor | None = None, start_iter: int = 0, residuals=None) -> SirtResult:
        """Iterate from x0 (zeros if None) until cfg.iters or the tolerance.
        residuals[k] holds ||b - A x|| / ||b|| of the x entering iteration k."""
        cfg = self.cfg
        x = torch.zeros(self._x_shape(), dtype=torch.float32, device=self.b.device) if x0 is None else x0
        x = x.contiguous()
        residuals = list(residuals or [])
        sync = torch.cuda.synchronize if x.is_cuda else (lambda: None)
        if cfg.use_graph:
            self.graph = self._capture(x)
        sync()
        t0 = time.perf_counter()
        it = start_iter
        while it < cfg.iters:
            if self.graph is not None:
                self.graph.replay()
            else:
                self._step(x)
            it += 1
            if it % cfg.check_every == 0 or it == cfg.iters:
                # the norms measure the residual of the x before this step's update
                r = relative_residual(self.norms)
                residuals.append((it, r))
                if cfg.tol > 0 and r <= cfg.tol:
                    break
            if cfg.checkpoint and cfg.checkpoint_every and it % cfg.checkpoint_every == 0:
                save_checkpoint(cfg.checkpoint, x, it, residuals)
        sync()
        self.x = x
        return SirtResult(x, it, residuals, time.perf_counter() - t0)

    def data_residual(self, x) -> float:
        """||b - A x|| / ||b|| of the current x."""
        norms = torch.zeros(2, dtype=torch.float64, device=x.device)
        self.plan.fp_residual(x, self.b, None, 0.0, out=self.e, norms=norms)
        return relative_residual(norms)


@dataclass
class AsdConfig:
    """SIRT-TV with the TV step tied to the data step (ASD-POCS, Sidky and Pan
    2008): every outer iteration runs one SIRT step, then ``tv_iters`` TV
    sub-steps whose RMS size is alpha * rms(SIRT change); alpha shrinks by
    ``alpha_red`` whenever the TV sub-steps moved x further than ``r_max`` times
    the SIRT step did.  As the data step shrinks so does the regulariser, so the
    data residual keeps falling (a fixed TV step stalls it)."""
    iters: int = 500
    lam: float = 1.0
    eps: float = 1e-9
    tv_iters: int = 20
    alpha: float = 0.2
    alpha_red: float = 0.95
    r_max: float = 0.95
    tv_eps: float = 1e-8
    tol: float = 0.0             # stop when ||b - A x|| / ||b|| <= tol


class AsdLoop:
    """SIRT3D + TV (AsdConfig) on one plan.  The row / column sums depend only
    on the geometry and are computed once; data and starting image are copied
    into fixed buffers, so one captured CUDA graph of an iteration serves every
    run.  The step sizes stay on the device: a run syncs only for residual
    checks."""

    def __init__(self, plan, cfg: AsdConfig | None = None, use_graph: bool = False):
        self.plan, self.cfg = plan, cfg or AsdConfig()
        g = plan.geom
        dev_ = torch.device("cuda")
        self.b = torch.zeros(g.sino_shape, dtype=torch.float32, device=dev_)
        self.s = Sirt(plan, self.b, SirtConfig(lam=self.cfg.lam, eps=self.cfg.eps))
        self.x = torch.zeros(g.vol_shape, dtype=torch.float32, device=dev_)
        self.prev = torch.empty_like(self.x)
        self.work = torch.empty_like(self.x)
        self.scratch = torch.zeros(2, dtype=torch.float64, device=dev_)
        self.state = torch.tensor([self.cfg.alpha, 0.0, 0.0], dtype=torch.float64, device=dev_)
        self.graph = None
        if use_graph:
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                self._step()                        # first call sets up plan workspaces
            torch.cuda.current_stream().wait_stream(side)
            torch.cuda.synchronize()
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph):
                self._step()

    def _step(self):
        c, s = self.cfg, self.s
        self.prev.copy_(self.x)
        s.norms.zero_()
        self.plan.fp_residual(self.x, self.b, s.rowsum, c.eps, out=s.e, norms=s.norms)
        self.plan.bp_update(s.e, s.colsum, self.x, lam=c.lam, eps=c.eps, lo=0.0, hi=float("inf"))
        if c.tv_iters > 0:
            dev.tv_flow_asd(self.x, self.prev, self.work, self.scratch, self.state, c.tv_iters, c.tv_eps, 0.0,
                            c.alpha_red, c.r_max)

    def run(self, b: torch.Tensor, x0: torch.Tensor, iters: int | None = None, tol: float | None = None,
            check_every: int = 1) -> SirtResult:
        """Iterate from x0 on data b.  residuals: (k, relative data residual of
        the x entering iteration k) at the checked iterations; times: seconds
        from the start (after the copies in) to each check.  result.x is a
        copy."""
        c = self.cfg
        iters = c.iters if iters is None else iters
        tol = c.tol if tol is None else tol
        self.b.copy_(b)
        self.x.copy_(x0)
        self.state[0] = c.alpha
        residuals, times = [], []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        it = 0
        while it < iters:
            if self.graph is not None:
                self.graph.replay()
            else:
                self._step()
            it += 1
            if it % check_every == 0 or it == iters:
                r = relative_residual(self.s.norms)
                residuals.append((it, r))
                times.append(time.perf_counter() - t0)
                if tol > 0 and r <= tol:
                    break
        torch.cuda.synchronize()
        res = SirtResult(self.x.clone(), it, residuals, time.perf_counter() - t0)
        res.alpha = float(self.state[0])
        res.times = times
        return res


def sirt_tv_asd(plan, b: torch.Tensor, x0: torch.Tensor, cfg: AsdConfig | None = None, check_every: int = 1,
                use_graph: bool = False) -> SirtResult:
    """SIRT3D + TV (AsdConfig) from x0 on data b (one AsdLoop run)."""
    return AsdLoop(plan, cfg, use_graph).run(b, x0, check_every=check_every)


def save_checkpoint(path, x: torch.Tensor, iteration: int, residuals):
    """SIRT state (x, iteration, residual history) as an .npz, written atomically."""
    path = Path(path)
    tmp = path.with_suffix(".tmp.npz")
    np.savez(tmp, x=x.detach().cpu().numpy(), iteration=np.int64(iteration),
             residuals=np.asarray(residuals, dtype=np.float64).reshape(-1, 2))
    tmp.replace(path)


def load_checkpoint(path, device="cuda"):
    d = np.load(path)
    res = [(int(i), float(r)) for i, r in d["residuals"]]
    return torch.from_numpy(d["x"]).to(device), int(d["iteration"]), res


def sirt3d(plan: dev.ConePlan, b, cfg: SirtConfig | None = None, x0=None) -> SirtResult:
    """SIRT3D (SIRT3D.m:67-92): lam 1, x >= 0, eps 1e-9, zero start."""
    cfg = cfg or SirtConfig()
    return Sirt(plan, b, cfg).run(x0)


def sirt_fan(plan: dev.FanPlan, b, cfg: SirtConfig | None = None, fbp_start: bool = True) -> SirtResult:
    """2D fan SIRT with the GPU operators (SIRT.m:99-144, :123-124, :131):
    lam 2, x in [0, 1], MATLAB eps, FBPfan start."""
    cfg = cfg or SirtConfig(iters=100, lam=2.0, lo=0.0, hi=1.0, eps=MATLAB_EPS)
    x0 = plan.fbp(b) if fbp_start else None   # the raw FBP image, as SIRT.m:109 starts
    return Sirt(plan, b, cfg).run(x0)


# -- metrics of the reference scripts ----------------------------------------
def rrmse(x, ref) -> float:
    """rRMSE.m: sqrt(mean((x - ref)^2)) / (sqrt(mean(ref^2)) + eps)."""
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.sqrt(np.mean((x - ref) ** 2)) / (np.sqrt(np.mean(ref ** 2)) + MATLAB_EPS))


def local_error(cur, prev) -> float:
    """LocalError.m: ||cur - prev|| / ||prev||."""
    cur = np.asarray(cur, np.float64)
    prev = np.asarray(prev, np.float64)
    return float(np.linalg.norm(cur - prev) / np.linalg.norm(prev))


def psnr(x, ref, peak: float = 1.0) -> float:
    mse = float(np.mean((np.asarray(x, np.float64) - np.asarray(ref, np.float64)) ** 2))
    return float("inf") if mse == 0 else 10.0 * math.log10(peak * peak / mse)
