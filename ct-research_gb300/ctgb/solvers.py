"""Reconstruction algorithms of the reference that call the projectors, on the
device-resident operators of this package.

* ``art`` -- ART / Kaczmarz on the exported system matrix (Iterative_algorithm/
  ART.m:57-75): one native row-action sweep per iteration (ct_csr_kaczmarz).
* ``cg`` -- the conjugate-gradient solver of Iterative_algorithm/cg.m.
* ``gradient2d_matrices``, ``soft_threshold``, ``cut`` and ``tv_cg`` -- the
  split-Bregman TV reconstruction of My_novel_algorithm/AdaptivePatch/TVCG.m
  (and the normal operator of TVpatchpriorPICCS.m:161): CG on
  mu A^T A (+ lambda div) with A the GPU projector, Sobel-type gradients with
  mirrored edges (gradient2Dmatrix_x.m / gradient2Dmatrix_y.m).
* ``hessian_log_templates``, ``hessian_log3d``, ``hstar_omega`` and
  ``hessian_schatten_tv`` -- the Hessian-Schatten TV reconstruction of
  My_novel_algorithm/HessianSchattenTV/HessianSchattenTV.m:93-175: an outer
  FP/BP data step through the cone operators and a Nesterov loop on the
  Hessian-Schatten dual (HessianLOG3D.m, HstarOmega.m, ObjectiveFunction.m,
  StopDeterminer.m).  Three places of those MATLAB files cannot run as
  written and are restated by their evident intent: HessianLOG3D convolves
  the 3-D image with the 5-D template H(i,j,:,:,:) (MATLAB's convn then acts
  along the template's leading singleton axes), HstarOmega adds 5-D
  convolutions to a 3-D array, and the Frobenius projection loops its first
  voxel index over all voxels.  Here both operators use the squeezed 3^3
  templates and the projection runs once per voxel.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib


# ---------------------------------------------------------------------------
# ART
# ---------------------------------------------------------------------------
def art(A, b: torch.Tensor, x0: torch.Tensor | None = None, lam: float = 0.3, sweeps: int = 5,
        lo: float | None = None, hi: float | None = None) -> torch.Tensor:
    """Kaczmarz sweeps over the rows of a CsrMatrix A (ctgb.device.CsrMatrix),
    rows in order: x <- x - lam a_j (a_j.x - b_j) / (a_j.a_j).  ART.m starts
    from zeros (ones for its MART variant); lo / hi clamp after each sweep."""
    rows, cols = A.shape
    x = torch.zeros(cols, dtype=torch.float32, device=b.device) if x0 is None else x0.reshape(-1).clone()
    b = b.reshape(-1).contiguous().float()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(sweeps):
        _lib.call("ct_csr_kaczmarz", C.c_void_p(A.row_ptr.data_ptr()), C.c_void_p(A.col.data_ptr()),
                  C.c_void_p(A.val.data_ptr()), C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), 0, rows,
                  float(lam), st)
        if lo is not None or hi is not None:
            x.clamp_(min=lo, max=hi)
    return x


# ---------------------------------------------------------------------------
# CG (cg.m)
# ---------------------------------------------------------------------------
@dataclass
class CGResult:
    x: torch.Tensor
    flag: int
    res_ne: float
    iterations: int


def cg(apply, b: torch.Tensor, tol: float = 1e-6, maxit: int | None = None, x0: torch.Tensor | None = None
       ) -> CGResult:
    """Conjugate gradients for a symmetric positive (semi-)definite operator
    given as a function, with cg.m's stopping rule and flags: 1 converged
    (|r| <= tol |r0|, or |x| tol >= 1), 2 maximum iterations, 3 indefinite,
    4 shrinking iterate; the later ones override the earlier as in cg.m."""
    if x0 is not None:
        x = x0.clone()
        r = b - apply(x)
    else:
        x = torch.zeros_like(b)
        r = b.clone()
    n = b.numel()
    if maxit is None:
        maxit = min(n, 20)
    p = r.clone()
    normr0 = float(torch.linalg.vector_norm(r))
    gamma = normr0 ** 2
    normx = float(torch.linalg.vector_norm(x))
    xmax = normx
    k, flag, indefinite, res_ne = 0, 0, False, 1.0
    while k < maxit and flag == 0:
        k += 1
        q = apply(p)
        delta = float(torch.dot(p.reshape(-1).double(), q.reshape(-1).double()))
        if delta <= 0:
            indefinite = True
        if delta == 0:
            delta = np.finfo(np.float64).eps
        alpha = gamma / delta
        x = x + alpha * p
        r = r - alpha * q
        normr = float(torch.linalg.vector_norm(r))
        gamma1, gamma = gamma, normr ** 2
        beta = gamma / gamma1 if gamma1 != 0 else 0.0
        p = r + beta * p
        normx = float(torch.linalg.vector_norm(x))
        xmax = max(xmax, normx)
        flag = int(normr <= normr0 * tol or normx * tol >= 1)
        res_ne = normr / normr0 if normr0 else 0.0
    if k == maxit:
        flag = 2
    if indefinite:
        flag = 3
    if xmax and normx / xmax <= math.sqrt(tol):
        flag = 4
    return CGResult(x, flag, res_ne, k)


# ---------------------------------------------------------------------------
# TV-CG (split Bregman)
# ---------------------------------------------------------------------------
def gradient2d_matrices(height: int, width: int):
    """Sobel-type gradients with mirrored edges as sparse matrices on pixel
    vectors (y-major, x fastest), exactly as gradient2Dmatrix_x.m and
    gradient2Dmatrix_y.m build them (row index (y-1)*height + x, 1-based)."""
    from scipy.sparse import coo_matrix

    def build(sobel, xsel, ysel):
        rows, cols, vals = [], [], []
        for x in range(1, width + 1):
            for y in range(1, height + 1):
                xi, yi = xsel(x), ysel(y)
                X, Y = np.meshgrid(xi, yi)            # MATLAB meshgrid, then transposed
                X, Y = X.T.ravel(order="F"), Y.T.ravel(order="F")
                for n in range(6):
                    rows.append((y - 1) * height + x - 1)
                    cols.append((y + Y[n] - 1) * width + (x + X[n]) - 1)
                    vals.append(sobel[n])
        return coo_matrix((vals, (rows, cols)), shape=(height * width, height * width)).tocsr()

    def edge2(i, n):
        return [0, 1] if i == 1 else ([-1, 0] if i == n else [-1, 1])

    def edge3(i, n):
        return [0, 0, 1] if i == 1 else ([-1, 0, 0] if i == n else [-1, 0, 1])

    gx = build([-1, 1, -2, 2, -1, 1], lambda x: edge2(x, width), lambda y: edge3(y, height))
    gy = build([-1, -2, -1, 1, 2, 1], lambda x: edge3(x, width), lambda y: edge2(y, height))
    return gx, gy


def soft_threshold(b: torch.Tensor, t: float) -> torch.Tensor:
    """soft_threshold.m: sign(b) max(|b| - t, 0)."""
    return torch.sign(b) * torch.clamp(b.abs() - t, min=0.0)


def cut(x: torch.Tensor, t: float) -> torch.Tensor:
    """Cut.m: x where |x| < t, +-t beyond (exactly +-t maps to 0, as Cut.m's branches leave it)."""
    out = torch.where(x.abs() < t, x, torch.zeros_like(x))
    out = torch.where(x > t, torch.full_like(x, t), out)
    return torch.where(x < -t, torch.full_like(x, -t), out)


def _torch_csr(m, device):
    m = m.tocsr()
    return torch.sparse_csr_tensor(torch.from_numpy(m.indptr.astype(np.int64)),
                                   torch.from_numpy(m.indices.astype(np.int64)),
                                   torch.from_numpy(m.data.astype(np.float64)), size=m.shape,
                                   dtype=torch.float64).to(device)


@dataclass
class TVCGResult:
    x: torch.Tensor
    loss: list = field(default_factory=list)
    local_error: list = field(default_factory=list)


def tv_cg(A, R: torch.Tensor, height: int, width: int, mu: float = 200.0, lam: float = 0.2, iter_cg: int = 80,
          outer: int = 20, inner: int = 10, threshold: float = 1e-6, lo: float = 0.0, hi: float = 1.0,
          x0: torch.Tensor | None = None, with_div: bool = False) -> TVCGResult:
    """Split-Bregman TV reconstruction of TVCG.m:46-93 with the projector A
    (a CsrMatrix; A^T is its transpose): each inner step solves
    mu A^T A x (+ lam div x when with_div) = mu A^T R by CG (warm start),
    clamps to [lo, hi], then updates (d, b) by soft thresholding and Cut of the
    Sobel gradients; inner steps stop on the relative change threshold."""
    import warnings
    dev = R.device
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", UserWarning)
        At = A.to_torch().to(torch.float64)
        gx, gy = gradient2d_matrices(height, width)
        Gx, Gy = _torch_csr(gx, dev), _torch_csr(gy, dev)
        Div = _torch_csr(gx.T @ gx + gy.T @ gy, dev)
    R = R.reshape(-1).double()
    ATt = At.t().to_sparse_csr()
    b1 = mu * torch.mv(ATt, R)

    def normal(v):
        out = mu * torch.mv(ATt, torch.mv(At, v))
        return out + lam * torch.mv(Div, v) if with_div else out

    x = torch.zeros(height * width, dtype=torch.float64, device=dev) if x0 is None else x0.reshape(-1).double()
    res = TVCGResult(x)
    thr = 1.0 / (lam + np.finfo(np.float64).eps)
    for _ in range(outer):
        bx = torch.zeros_like(x)
        by = torch.zeros_like(x)
        local_e, it = 100.0, 1
        while it <= inner and local_e > threshold:
            prev = x
            x = cg(normal, b1, tol=1e-6, maxit=iter_cg, x0=prev).x.clamp(lo, hi)
            gxx, gyx = torch.mv(Gx, x), torch.mv(Gy, x)
            bx = cut(gxx + bx, thr)
            by = cut(gyx + by, thr)
            local_e = float(torch.linalg.vector_norm(x - prev) / (torch.linalg.vector_norm(prev) + 1e-10))
            res.local_error.append(local_e)
            res.loss.append(float(gxx.abs().sum() + gyx.abs().sum()
                                  + 0.5 * mu * torch.linalg.vector_norm(torch.mv(At, x) - R)))
            it += 1
    res.x = x
    return res


# ---------------------------------------------------------------------------
# Hessian-Schatten TV
# ---------------------------------------------------------------------------
def hessian_log_templates(ps: int = 3, device="cpu") -> torch.Tensor:
    """HessianLOGtemplate3D.m: the 3 x 3 matrix of LoG second-derivative
    templates (sigma 1) on a ps^3 patch, indices (i, j, k) on axes (x, y, z)
    with x = i - (ps - 1)/2 for i = 1..ps."""
    H = np.zeros((3, 3, ps, ps, ps))
    s = 1.0
    c0 = -1.0 / ((2 * math.pi) ** 3 * s ** 5)
    c1 = 1.0 / ((2 * math.pi) ** 3 * s ** 7)
    for i in range(1, ps + 1):
        for j in range(1, ps + 1):
            for k in range(1, ps + 1):
                x, y, z = i - (ps - 1) / 2, j - (ps - 1) / 2, k - (ps - 1) / 2
                e = math.exp(-(x * x + y * y + z * z) / (2 * s * s))
                hx = c0 * (1 - x * x / s ** 2) * e
                hy = c0 * (1 - y * y / s ** 2) * e
                hz = c0 * (1 - z * z / s ** 2) * e
                hxy, hxz, hyz = c1 * x * y * e, c1 * x * z * e, c1 * y * z * e
                H[:, :, i - 1, j - 1, k - 1] = [[hx, hxy, hxz], [hxy, hy, hyz], [hxz, hyz, hz]]
    return torch.from_numpy(H).to(device)


def _convn_same(u: torch.Tensor, kern: torch.Tensor) -> torch.Tensor:
    """MATLAB convn(u, kern, 'same') on a 3D array (true convolution, zero padded)."""
    import torch.nn.functional as F
    ps = kern.shape[-1]
    k = torch.flip(kern, dims=(-3, -2, -1)).reshape(1, 1, ps, ps, ps)
    pad = ps // 2
    return F.conv3d(u.reshape(1, 1, *u.shape), k.to(u.dtype), padding=pad)[0, 0]


def hessian_log3d(u: torch.Tensor, H: torch.Tensor) -> torch.Tensor:
    """HessianLOG3D.m: the 3 x 3 Hessian field of the 3D array u (axes x, y, z
    as MATLAB's dims 1, 2, 3), shape (3, 3, *u.shape)."""
    out = torch.empty((3, 3, *u.shape), dtype=u.dtype, device=u.device)
    for i in range(3):
        for j in range(3):
            out[i, j] = _convn_same(u, H[i, j])
    return out


def hstar_omega(omega: torch.Tensor, H: torch.Tensor) -> torch.Tensor:
    """HstarOmega.m: sum_ij convn(omega_ij, H_ij with its first and last planes
    swapped along each axis, 'same') -- for the 3^3 templates a full flip, so
    this is the adjoint of hessian_log3d."""
    ps = H.shape[-1]
    if ps != 3:
        raise ValueError("HstarOmega's plane swap is defined for 3^3 templates")
    Ht = torch.flip(H, dims=(2, 3, 4))
    out = torch.zeros(omega.shape[2:], dtype=omega.dtype, device=omega.device)
    for i in range(3):
        for j in range(3):
            out += _convn_same(omega[i, j], Ht[i, j])
    return out


def schatten_norm(hs: torch.Tensor, order: int = 2) -> torch.Tensor:
    """Sum over voxels of the Schatten-p norm of the 3 x 3 Hessians (ObjectiveFunction.m)."""
    m = hs.permute(*range(2, hs.dim()), 0, 1).reshape(-1, 3, 3)
    sv = torch.linalg.svdvals(m)
    return (sv ** order).sum(dim=1).pow(1.0 / order).sum()


def stop_determiner(cur: torch.Tensor, prev: torch.Tensor, threshold: float) -> bool:
    """StopDeterminer.m: ||cur - prev|| / (||prev|| + 1e-10) <= threshold."""
    return float(torch.linalg.vector_norm(cur - prev) / (torch.linalg.vector_norm(prev) + 1e-10)) <= threshold


@dataclass
class HSTVResult:
    x: torch.Tensor
    objective: list = field(default_factory=list)
    outer_iterations: int = 0


def hessian_schatten_tv(plan, V: torch.Tensor, u0: torch.Tensor, alpha: float = 2e2, tau: float = 1.0,
                        order: int = 2, outer: int = 40, inner: int = 30, outer_threshold: float = 1e-3,
                        inner_threshold: float = 1e-3, ps: int = 3) -> HSTVResult:
    """HessianSchattenTV.m:93-175 on a ConePlan: majorisation-minimisation
    outer loop Z = X + BP(V - FP(X)) / alpha (FP = ProjectionCone_3D,
    BP = Backprojection), a Nesterov loop on the dual Omega (projection on the
    Frobenius unit ball per voxel, order 2), S = Z - tau H*(Omega), a monotone
    choice of U by the objective, and the FISTA extrapolation of X."""
    H = hessian_log_templates(ps, V.device).to(torch.float64)
    L = 144 * tau ** 2
    shape = u0.shape

    def objective(u):
        r = V - plan.fp(u.float())
        return 0.5 * float(torch.sum(r.double() ** 2)) + tau * float(schatten_norm(hessian_log3d(u.double(), H), order))

    res = HSTVResult(u0)
    k_mm_prev = 1.0
    c_prev = objective(u0)
    res.objective.append(c_prev)
    u_prev = u0.double()
    x_prev = u0.double()
    zero = torch.zeros((3, 3, *shape), dtype=torch.float64, device=V.device)
    for t in range(outer):
        resid = V - plan.fp(x_prev.float())
        z = x_prev + plan.bp(resid.contiguous()).double() / alpha
        kn_prev = 1.0
        pbs_prev, om_prev = zero.clone(), zero.clone()
        for _ in range(inner):
            prn = z - tau * hstar_omega(om_prev, H)
            pbs = om_prev + tau * hessian_log3d(prn, H) / L
            if order == 2:
                fro = torch.sqrt((pbs ** 2).sum(dim=(0, 1)))
                pbs = pbs / torch.clamp(fro, min=1.0)
            kn = (1 + math.sqrt(1 + kn_prev ** 2)) / 2
            om = pbs_prev + (kn_prev - 1) / kn * (pbs - pbs_prev)
            if stop_determiner(pbs, pbs_prev, inner_threshold):
                break
            kn_prev, om_prev, pbs_prev = kn, om, pbs
        s = z - tau * hstar_omega(pbs_prev, H)
        k_mm = (1 + math.sqrt(1 + k_mm_prev ** 2)) / 2
        c_cur = objective(s)
        u_cur = u_prev if c_cur > c_prev else s
        x_cur = u_cur + (k_mm_prev / k_mm) * (s - u_cur) + (k_mm_prev - 1) / k_mm * (u_cur - u_prev)
        res.objective.append(c_cur if c_cur <= c_prev else c_prev)
        res.outer_iterations = t + 1
        if stop_determiner(u_cur, u_prev, outer_threshold):
            u_prev = u_cur
            break
        u_prev, c_prev, x_prev, k_mm_prev = u_cur, c_cur, x_cur, k_mm
    res.x = u_prev
    return res
