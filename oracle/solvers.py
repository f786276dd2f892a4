"""The reference's MATLAB reconstruction loops that call the projectors, restated
in numpy float64 (TEST INFRASTRUCTURE ONLY: the checker of ctgb.solvers).

* ``tvcg`` -- the split-Bregman TV reconstruction of
  My_novel_algorithm/AdaptivePatch/TVCG.m:58-142 with its helpers cg.m
  (Iterative_algorithm/cg.m:84-165), soft_threshold.m, Cut.m, LocalError.m and
  gradient2Dmatrix_x.m / gradient2Dmatrix_y.m (My_toolbox/), line by line.
* ``hessian_schatten_tv`` -- My_novel_algorithm/HessianSchattenTV/
  HessianSchattenTV.m:66-175 with HessianLOGtemplate3D.m, HessianLOG3D.m,
  HstarOmega.m, ObjectiveFunction.m and StopDeterminer.m.  The data step calls
  the given projector / backprojector (the oracle's restatements of the
  reference kernels in the tests).  Three places of those files cannot run as
  written and are restated by their evident intent, as the product does:
  HessianLOG3D convolves the 3-D image with the squeezed 3^3 template,
  HstarOmega sums 3-D convolutions of the squeezed dual components, and the
  Frobenius projection visits every voxel once.

Nothing here is imported by the product path.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.ndimage import convolve

EPS = 2.220446049250313e-16        # MATLAB eps


# -- TVCG.m and its helpers ----------------------------------------------------
def cg(afun, b, tol=1e-6, maxit=None, x0=None):
    """cg.m with a function handle: returns (x, flag, resNE, iter)."""
    if x0 is not None:
        x = np.array(x0, dtype=np.float64)
        r = b - afun(x)
    else:
        r = b.copy()
        x = np.zeros_like(b)
    m = n = b.shape[0]
    if maxit is None:
        maxit = min(m, n, 20)
    p = r.copy()
    normr0 = np.linalg.norm(r)
    gamma = normr0 ** 2
    normx = np.linalg.norm(x)
    xmax = normx
    k, flag, indefinite, res_ne = 0, 0, 0, 1.0
    while k < maxit and flag == 0:
        k += 1
        q = afun(p)
        delta = p @ q
        if delta <= 0:
            indefinite = 1
        if delta == 0:
            delta = EPS
        alpha = gamma / delta
        x = x + alpha * p
        r = r - alpha * q
        normr = np.linalg.norm(r)
        gamma1 = gamma
        gamma = normr ** 2
        beta = gamma / gamma1
        p = r + beta * p
        normx = np.linalg.norm(x)
        xmax = max(xmax, normx)
        flag = int(normr <= normr0 * tol or normx * tol >= 1)
        res_ne = normr / normr0
    shrink = normx / xmax
    if k == maxit:
        flag = 2
    if indefinite:
        flag = 3
    if shrink <= math.sqrt(tol):
        flag = 4
    return x, flag, res_ne, k


def soft_threshold(b, t):
    """soft_threshold.m"""
    return np.sign(b) * np.maximum(np.abs(b) - t, 0)


def cut(v, t):
    """Cut.m, element by element (an entry equal to +-t becomes 0)."""
    out = np.zeros(len(v))
    for i in range(len(v)):
        if abs(v[i]) < t:
            out[i] = v[i]
        elif v[i] > t:
            out[i] = t
        elif v[i] < -t:
            out[i] = -t
    return out


def local_error(cur, prev):
    """LocalError.m"""
    return np.linalg.norm(cur - prev) / np.linalg.norm(prev)


def _gradient_matrix(height, width, sobel, xsel, ysel):
    from scipy.sparse import coo_matrix
    rows, cols, w = [], [], []
    for x in range(1, width + 1):
        for y in range(1, height + 1):
            xi, yi = np.meshgrid(xsel(x), ysel(y))
            xi, yi = xi.T, yi.T                         # xindex', yindex'
            xi, yi = xi.ravel(order="F"), yi.ravel(order="F")
            for n in range(6):
                rows.append((y - 1) * height + x)
                cols.append((y + yi[n] - 1) * width + (x + xi[n]))
                w.append(sobel[n])
    return coo_matrix((w, (np.array(rows) - 1, np.array(cols) - 1)), shape=(height * width, height * width)).tocsr()


def gradient2d_x(height, width):
    """gradient2Dmatrix_x.m"""
    return _gradient_matrix(height, width, [-1, 1, -2, 2, -1, 1],
                            lambda x: [0, 1] if x == 1 else ([-1, 0] if x == width else [-1, 1]),
                            lambda y: [0, 0, 1] if y == 1 else ([-1, 0, 0] if y == height else [-1, 0, 1]))


def gradient2d_y(height, width):
    """gradient2Dmatrix_y.m"""
    return _gradient_matrix(height, width, [-1, -2, -1, 1, 2, 1],
                            lambda x: [0, 0, 1] if x == 1 else ([-1, 0, 0] if x == width else [-1, 0, 1]),
                            lambda y: [0, 1] if y == 1 else ([-1, 0] if y == height else [-1, 1]))


def tvcg(A, R, height, width, miu=200.0, lamda1=0.2, iter_cg=80, outeriter=20, inner=10, threshold=1e-6,
         lo=0.0, hi=1.0):
    """TVCG.m:58-142: returns (Display vector, list of loss values)."""
    A = A.tocsr()
    At = A.T.tocsr()
    gx, gy = gradient2d_x(height, width), gradient2d_y(height, width)
    b1 = miu * (At @ R)
    display_prev = np.zeros(height * width)
    losses = []
    display = display_prev
    for _ in range(outeriter):
        display = display_prev.copy()
        bx1 = np.zeros(height * width)
        by1 = np.zeros(height * width)
        local_e, it = 100.0, 1
        while it <= inner and local_e > threshold:
            display_prev = display
            display, _, _, _ = cg(lambda v: miu * (At @ (A @ v)), b1, 1e-6, iter_cg, display_prev)
            display = np.clip(display, lo, hi)
            t = 1.0 / (lamda1 + EPS)
            bx1 = cut(gx @ display + bx1, t)
            by1 = cut(gy @ display + by1, t)
            with np.errstate(divide="ignore", invalid="ignore"):
                local_e = local_error(display, display_prev)
            losses.append(np.abs(gx @ display).sum() + np.abs(gy @ display).sum()
                          + 0.5 * miu * np.linalg.norm(A @ display - R))
            it += 1
        display_prev = display
    return display, losses


# -- HessianSchattenTV.m and its helpers ---------------------------------------
def hessian_log_template3d(ps=3):
    """HessianLOGtemplate3D.m: H[i, j, x, y, z], LoG second derivatives, sigma 1."""
    H = np.zeros((3, 3, ps, ps, ps))
    s = 1.0
    for i in range(1, ps + 1):
        for j in range(1, ps + 1):
            for k in range(1, ps + 1):
                x, y, z = i - (ps - 1) / 2, j - (ps - 1) / 2, k - (ps - 1) / 2
                e = math.exp(-(x * x + y * y + z * z) / (2 * s * s))
                a = -1 / ((2 * math.pi) ** 3 * s ** 5)
                b = 1 / ((2 * math.pi) ** 3 * s ** 7)
                H[0, 0, i - 1, j - 1, k - 1] = a * (1 - x * x / s ** 2) * e
                H[1, 1, i - 1, j - 1, k - 1] = a * (1 - y * y / s ** 2) * e
                H[2, 2, i - 1, j - 1, k - 1] = a * (1 - z * z / s ** 2) * e
                H[0, 1, i - 1, j - 1, k - 1] = H[1, 0, i - 1, j - 1, k - 1] = b * x * y * e
                H[0, 2, i - 1, j - 1, k - 1] = H[2, 0, i - 1, j - 1, k - 1] = b * x * z * e
                H[1, 2, i - 1, j - 1, k - 1] = H[2, 1, i - 1, j - 1, k - 1] = b * y * z * e
    return H


def _convn_same(u, k):
    """MATLAB convn(u, k, 'same') for odd k: zero padding, the kernel flipped."""
    return convolve(u, k, mode="constant", cval=0.0)


def hessian_log3d(u, H):
    """HessianLOG3D.m: (3, 3, Lx, Ly, Lz)."""
    out = np.zeros((3, 3) + u.shape)
    for i in range(3):
        for j in range(3):
            out[i, j] = _convn_same(u, H[i, j])
    return out


def hstar_omega(omega, H, ps=3):
    """HstarOmega.m: the templates with planes 1..num and ps-num+1 swapped along
    each axis (num = ceil((ps - 1) / 2)), then sum_ij convn(omega_ij, Ht_ij)."""
    Ht = H.copy()
    num = math.ceil((ps - 1) / 2)
    for ax in (2, 3, 4):
        a = np.take(Ht, range(num), axis=ax).copy()
        sl_lo = [slice(None)] * 5
        sl_hi = [slice(None)] * 5
        sl_lo[ax] = slice(0, num)
        sl_hi[ax] = slice(ps - num, ps - num + 1)
        Ht[tuple(sl_lo)] = Ht[tuple(sl_hi)]
        Ht[tuple(sl_hi)] = a
    out = np.zeros(omega.shape[2:])
    for i in range(ps):
        for j in range(ps):
            out += _convn_same(omega[i, j], Ht[i, j])
    return out


def objective_function(V, AU, U, order, tau, H):
    """ObjectiveFunction.m"""
    hs = hessian_log3d(U, H)
    m = np.moveaxis(hs.reshape(3, 3, -1), -1, 0)
    sv = np.linalg.svd(m, compute_uv=False)
    hsnorm = float(np.sum(np.sum(sv ** order, axis=1) ** (1.0 / order)))
    r = (V - AU).ravel()
    return 0.5 * float(r @ r) + tau * hsnorm


def stop_determiner(cur, prev, threshold):
    """StopDeterminer.m"""
    return np.linalg.norm((cur - prev).ravel()) / (np.linalg.norm(prev.ravel()) + 1e-10) <= threshold


def hessian_schatten_tv(fp, bp, V, U0, alpha=2e2, tau=1.0, order=2, tmm=40, tnesterov=30, outer_threshold=1e-3,
                        inner_threshold=1e-3, ps=3):
    """HessianSchattenTV.m:66-175: fp / bp take and return float64 arrays
    (the script feeds them single precision: both round to float32 on the
    way in).  Returns (U, objective values of the accepted iterates, outer
    iterations run)."""
    H = hessian_log_template3d(ps)
    L = 144 * tau ** 2
    f32 = lambda a: np.asarray(a, np.float32)
    cfai_prev = objective_function(V, fp(f32(U0)), U0, order, tau, H)
    objective = [cfai_prev]
    u_prev = x_prev = np.asarray(U0, np.float64)
    kmm_prev = 1.0
    zero = np.zeros((3, 3) + U0.shape)
    t_run = 0
    u_cur = u_prev
    for t in range(tmm):
        t_run = t + 1
        resid = f32(V - fp(f32(x_prev)))
        z = x_prev + bp(resid) / alpha
        kn_prev = 1.0
        pbs_prev = zero.copy()
        om_prev = zero.copy()
        for _ in range(tnesterov):
            prn = z - tau * hstar_omega(om_prev, H, ps)
            pbs = om_prev + tau * hessian_log3d(prn, H) / L
            if order == 2:
                fro = np.sqrt((pbs ** 2).sum(axis=(0, 1)))
                pbs = np.where(fro > 1, pbs / np.where(fro > 1, fro, 1.0), pbs)
            kn = (1 + math.sqrt(1 + kn_prev ** 2)) / 2
            om = pbs_prev + (kn_prev - 1) / kn * (pbs - pbs_prev)
            if stop_determiner(pbs, pbs_prev, inner_threshold):
                break
            kn_prev, om_prev, pbs_prev = kn, om, pbs
        s = z - tau * hstar_omega(pbs_prev, H, ps)
        AS = fp(f32(s))
        kmm = (1 + math.sqrt(1 + kmm_prev ** 2)) / 2
        cfai = objective_function(V, AS, s, order, tau, H)
        u_cur = u_prev if cfai > cfai_prev else s
        x_cur = u_cur + (kmm_prev / kmm) * (s - u_cur) + (kmm_prev - 1) / kmm * (u_cur - u_prev)
        objective.append(min(cfai, cfai_prev))
        if stop_determiner(u_cur, u_prev, outer_threshold):
            break
        u_prev, cfai_prev, x_prev, kmm_prev = u_cur, cfai, x_cur, kmm
    return u_cur, objective, t_run
