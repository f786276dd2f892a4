"""MATLAB system-matrix builders restated in Python (TEST INFRASTRUCTURE ONLY).

GenSysMatFan.m and GenSysMatParal.m (Projection_computation_matlab/) walk each
ray with Siddon2D.m and collect sparse(L, J, W): row = ray in [beta][P] order,
column = pixel (y - 1) * width + x, value = the piece of the line between two
consecutive grid crossings.  The restatement follows those files step by step
(pure Python loops: small cases only) and returns scipy CSR matrices with
0-based indices, duplicates summed and zeros dropped as MATLAB's sparse() does.
It pins the GPU export (ct_fan_sysmat) to the reference's own matrix builder.
"""
from __future__ import annotations

import math

import numpy as np

EPS = 2.220446049250313e-16        # MATLAB eps


def _rangelimit(v):
    """rangelimit.m"""
    return 1e16 if v > 1e16 else (-1e16 if v < -1e16 else v)


def siddon2d(ys0, xs0, ye, xe, res, size, height, width, smax):
    """Siddon2D.m:12-99: crossings of the line (xs0, ys0) -> (xe, ye) with the
    grid lines, as columns (parameter * 2 smax, grid index, 1 = y / 2 = x),
    sorted (sortrows)."""
    xsl, xsr = math.floor(xs0 / res), math.ceil(xs0 / res)
    ysl, ysr = math.floor(ys0 / res), math.ceil(ys0 / res)
    xel, xer = math.floor(xe / res), math.ceil(xe / res)
    yel, yer = math.floor(ye / res), math.ceil(ye / res)
    if yer == ysr or yel == ysl:
        y_range, ysig = [], 0
    else:
        if ye > ys0:
            ysig = 1
            ystart = 0 if ys0 < 0 else ysl
            yend = height if ye > size[0] else yer
        else:
            ysig = -1
            ystart = 0 if ye < 0 else yel
            yend = height if ys0 > size[0] else ysr
        y_range = list(range(ystart, yend + 1))
    if xer == xsr or xel == xsl:
        x_range, xsig = [], 0
    else:
        if xe > xs0:
            xsig = 1
            xstart = 0 if xs0 < 0 else math.floor(xs0 / res)
            xend = width if xe > size[1] else math.ceil(xe / res)
        else:
            xsig = -1
            xstart = 0 if xe < 0 else math.floor(xe / res)
            xend = width if xs0 > size[1] else math.ceil(xs0 / res)
        x_range = list(range(xstart, xend + 1))
    cols = [(abs((y * res - ys0) / (ye - ys0)) * 2 * smax, y, 1) for y in y_range]
    cols += [(abs((x * res - xs0) / (xe - xs0)) * 2 * smax, x, 2) for x in x_range]
    cols.sort()
    return len(x_range), len(y_range), xsig, ysig, cols


def _walk(sys_rows, row, xs0, ys0, xe, ye, res, size, height, width, smax):
    """The pixel tracking loop shared by GenSysMatFan.m:33-87 and GenSysMatParal.m:36-70
    (both loop over every crossing; the last one leaves the image)."""
    lx, ly, xsig, ysig, pl = siddon2d(ys0, xs0, ye, xe, res, size, height, width, smax)
    if len(pl) <= 1:
        return
    x2y = _rangelimit((ye - ys0) / (xe - xs0 + EPS))
    y2x = _rangelimit((xe - xs0) / (ye - ys0 + EPS))
    dpx = dpy = None
    if pl[0][2] == 1:
        dpx = math.ceil((xs0 + (pl[0][1] * res - ys0) * y2x) / res)
    else:
        dpy = math.ceil((ys0 + (pl[0][1] * res - xs0) * x2y) / res)
    for n in range(len(pl)):
        if pl[n][2] == 1 and ly != 0:
            dpy = pl[n][1] + 0.5 + ysig * 0.5
        elif pl[n][2] == 2 and lx != 0:
            dpx = pl[n][1] + 0.5 + xsig * 0.5
        if dpy is not None and dpx is not None and 0 < dpy <= height and 0 < dpx <= width:
            if n + 1 >= len(pl):
                raise RuntimeError("the MATLAB loop would index past the last crossing")
            col = int((dpy - 1) * width + dpx) - 1
            sys_rows.append((row, col, pl[n + 1][0] - pl[n][0]))


def _csr(entries, nrows, ncols):
    from scipy.sparse import coo_matrix
    if not entries:
        return coo_matrix((nrows, ncols)).tocsr()
    r, c, w = (np.asarray(a) for a in zip(*entries))
    m = coo_matrix((w.astype(np.float64), (r, c)), shape=(nrows, ncols)).tocsr()   # sums duplicates
    m.eliminate_zeros()
    m.sort_indices()
    return m


def gensysmat_fan(height, width, size, beta, P, rscan, cx, cy):
    """GenSysMatFan.m:6-89 (size = [Size_y, Size_x])."""
    res = max(size) / height
    smax = 2 * rscan
    out = []
    for bi, b in enumerate(beta):
        sx = cx + rscan * math.sin(-b)
        sy = cy + rscan * math.cos(b)
        for pi_, p in enumerate(P):
            th = math.atan(p / rscan)
            ex = cx + smax * math.sin(th) * math.cos(-b) + (rscan - smax * math.cos(th)) * math.sin(-b)
            ey = cy - smax * math.sin(th) * math.sin(-b) + (rscan - smax * math.cos(th)) * math.cos(-b)
            _walk(out, bi * len(P) + pi_, sx, sy, ex, ey, res, size, height, width, rscan)
    return _csr(out, len(beta) * len(P), height * width)


def gensysmat_paral(height, width, size, cx, cy, theta, t_range):
    """GenSysMatParal.m:6-74."""
    res = max(size) / height
    smax = t_range[-1]
    out = []
    for ti, th in enumerate(theta):
        for k, t in enumerate(t_range):
            xs0 = cx + t * math.cos(-th) - smax * math.sin(-th)
            ys0 = cy - t * math.sin(-th) - smax * math.cos(-th)
            xe = cx + t * math.cos(-th) + smax * math.sin(-th)
            ye = cy - t * math.sin(-th) + smax * math.cos(-th)
            _walk(out, ti * len(t_range) + k, xs0, ys0, xe, ye, res, size, height, width, smax)
    return _csr(out, len(theta) * len(t_range), height * width)
