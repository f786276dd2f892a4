"""MATLAB-level operator API: the eight CT-Research MEX operators.

Each function takes the arguments of the reference's mexFunction in the same
order, with the same meaning and types, and returns what the gateway returns:
a float64 column vector (here a 1-D numpy array) of length L (volume or
sinogram size), in the reference layouts:

  ProjectionCone_3D(pic, t, s, z, Size, BetaScanRange, Pdomain, Xigamadomain, Distance)
      ProjectionCone_3D.cpp:5-36  -> sinogram [beta][xi][P]
  Backprojection3D(R, Xigamadomain, Pdomain, BetaScanRange, Distance, Size, t, s, z)
      Backprojection3D.cpp:7-34 (called ``Backprojection`` by the MATLAB scripts)
  FDK(R, Xigamadomain, Pdomain, BetaScanRange, Distance, Size, t, s, z)        FDK.cpp:7-40
  ProjectionFan_2D(pic, t, s, Size, BetaScanRange, Pdomain, Distance)         ProjectionFan_2D.cpp:5-30
  ProjectionParallel_2D(pic, height, width, Size, thetaRange, t_range)        ProjectionParallel_2D.cpp:5-28
  BackprojectionFan2D(R, BetaScanRange, Pdomain, Size, t, s, Rscan)          BackprojectionFan2D.cpp:7-39
  FBPfan(R, BetaScanRange, Pdomain, Size, t, s, Rscan)                       FBPfan.cpp:7-40
  FBPparallel(R, ThetaScanRange, Tdomain, Size, t, s)                        FBPparallel.cpp:7-38
  IterativeFDKerrCompute(Pic, t, s, z, Size, BetaScanRange, Udomain, Pdomain, Distance, G, t_slice)
      IterativeFDKerrCompute.cpp:3-58 -> error slice [beta][z][s]
  ImplementUI(R, Xigamadomain, Gamadomain, BetaScanRange, StartAngle, GamaMax, Distance, Distance_s2d, Size, z_length)
      ImplementUI.cpp:3-58 -> curved-detector FDK display [z][s][t]

Domain vectors are read with their length as MATLAB's mxGetM would (any
1-D array-like).  Single-precision arguments are converted to float32 and
double ones to float64, as the gateway's pointer casts assume.

Errors: the reference gateway prints a message and returns a zero-filled
output (ProjectionCone_3D.cpp:38-42).  Here a failure raises CTError with the
library's message; pass ``on_error="zeros"`` for the reference behaviour.
"""
from __future__ import annotations

import ctypes as C
import sys

import numpy as np

from . import _lib


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel())


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel())


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _run(name, out, on_error, *args):
    st = getattr(_lib.lib(), name)(*args)
    if st != 0:
        msg = _lib.lib().ct_last_error().decode(errors="replace")
        if on_error == "zeros":
            print(f"{name} failed: {msg}", file=sys.stderr)
            out[:] = 0
        else:
            raise _lib.CTError(st, name, msg)
    return out


def ProjectionCone_3D(pic, t_length, s_length, z_length, Size, BetaScanRange, Pdomain, Xigamadomain, Distance,
                      on_error="raise"):
    pic = _f32(pic)
    t, s, z = int(t_length), int(s_length), int(z_length)
    Size = _f64(Size)
    beta, P, xi = _f32(BetaScanRange), _f32(Pdomain), _f32(Xigamadomain)
    if pic.size != t * s * z:
        raise ValueError("pic must hold t_length*s_length*z_length values")
    res = _f64([Size[0] / t, Size[1] / s, Size[2] / z])
    out = np.zeros(len(beta) * len(P) * len(xi), np.float32)
    _run("ct_ProjectionCone_3D", out, on_error, _ptr(pic), _ptr(out), _ptr(beta), _ptr(P), _ptr(xi), t, s, z,
         Size[0] / 2, Size[1] / 2, Size[2] / 2, len(beta), len(P), len(xi), float(Distance), _ptr(res))
    return out.astype(np.float64)


def _bp3d(name, R, Xigamadomain, Pdomain, BetaScanRange, Distance, Size, t_length, s_length, z_length, on_error):
    R = _f32(R)
    xi, P, beta = _f32(Xigamadomain), _f32(Pdomain), _f32(BetaScanRange)
    Size = _f64(Size)
    t, s, z = int(t_length), int(s_length), int(z_length)
    if R.size != len(beta) * len(P) * len(xi):
        raise ValueError("R must hold LBeta*LP*LXigama values")
    out = np.zeros(t * s * z, np.float32)
    _run(name, out, on_error, _ptr(out), _ptr(R), _ptr(xi), _ptr(P), _ptr(beta), float(Distance), len(beta),
         len(P), len(xi), _ptr(Size), t, s, z)
    return out.astype(np.float64)


def Backprojection3D(R, Xigamadomain, Pdomain, BetaScanRange, Distance, Size, t_length, s_length, z_length,
                     on_error="raise"):
    return _bp3d("ct_BackPro", R, Xigamadomain, Pdomain, BetaScanRange, Distance, Size, t_length, s_length,
                 z_length, on_error)


Backprojection = Backprojection3D   # the name the MATLAB scripts use (HessianSchattenTV.m:101)


def FDK(R, Xigamadomain, Pdomain, BetaScanRange, Distance, Size, t_length, s_length, z_length, on_error="raise"):
    return _bp3d("ct_FDKpro", R, Xigamadomain, Pdomain, BetaScanRange, Distance, Size, t_length, s_length,
                 z_length, on_error)


def ProjectionFan_2D(pic, t_length, s_length, Size, BetaScanRange, Pdomain, Distance, on_error="raise"):
    pic = _f32(pic)
    t, s = int(t_length), int(s_length)
    Size = _f64(Size)
    beta, P = _f64(BetaScanRange), _f64(Pdomain)
    if pic.size != t * s:
        raise ValueError("pic must hold t_length*s_length values")
    res = _f64([Size[0] / t, Size[1] / s])
    out = np.zeros(len(beta) * len(P), np.float64)
    _run("ct_ProjectionFan_2D", out, on_error, _ptr(pic), _ptr(out), _ptr(beta), _ptr(P), t, s, Size[0] / 2,
         Size[1] / 2, len(beta), len(P), float(Distance), _ptr(res))
    return out


def ProjectionParallel_2D(pic, height, width, Size, thetaRange, t_range, on_error="raise"):
    pic = _f32(pic)
    h, w = int(height), int(width)
    Size = _f64(Size)
    th, tr = _f64(thetaRange), _f64(t_range)
    if pic.size != h * w:
        raise ValueError("pic must hold height*width values")
    res = _f64([Size[0] / h, Size[1] / w])
    out = np.zeros(len(th) * len(tr), np.float64)
    _run("ct_ProjectionParallel_2D", out, on_error, _ptr(pic), _ptr(out), _ptr(th), _ptr(tr), h, w, Size[0] / 2,
         Size[1] / 2, len(th), len(tr), _ptr(res))
    return out


def _bp2d(name, R, BetaScanRange, Pdomain, Size, t_length, s_length, Rscan, on_error):
    R = _f32(R)
    beta, P = _f32(BetaScanRange), _f32(Pdomain)
    Size = _f64(Size)
    t, s = int(t_length), int(s_length)
    if R.size != len(beta) * len(P):
        raise ValueError("R must hold LBeta*LP values")
    out = np.zeros(t * s, np.float32)
    if Rscan is None:
        _run(name, out, on_error, _ptr(out), _ptr(R), _ptr(P), _ptr(beta), len(beta), len(P), _ptr(Size), t, s)
    else:
        _run(name, out, on_error, _ptr(out), _ptr(R), _ptr(P), _ptr(beta), len(beta), len(P), _ptr(Size), t, s,
             float(Rscan))
    return out.astype(np.float64)


def BackprojectionFan2D(R, BetaScanRange, Pdomain, Size, t_length, s_length, Rscan, on_error="raise"):
    return _bp2d("ct_BackprojectionFan2D", R, BetaScanRange, Pdomain, Size, t_length, s_length, Rscan, on_error)


def FBPfan(R, BetaScanRange, Pdomain, Size, t_length, s_length, Rscan, on_error="raise"):
    return _bp2d("ct_FBPfan", R, BetaScanRange, Pdomain, Size, t_length, s_length, Rscan, on_error)


def FBPparallel(R, ThetaScanRange, Tdomain, Size, t_length, s_length, on_error="raise"):
    return _bp2d("ct_FBPpara", R, ThetaScanRange, Tdomain, Size, t_length, s_length, None, on_error)


# MATLAB layout helpers (My_toolbox/MatlabCpp_ImgVecTran_function)
def Img2vec_Mat2Cpp2D(img):
    """single(reshape(fliplr(Img'), numel(Img), 1)) for a MATLAB (column-major) image."""
    img = np.asarray(img)
    return np.asarray(np.fliplr(img.T), dtype=np.float32).ravel(order="F")


def Vec2img_Cpp2Mat2D(vec, height, width):
    """fliplr(reshape(vec, height, width))' -- inverse of Img2vec_Mat2Cpp2D."""
    m = np.asarray(vec).reshape((height, width), order="F")
    return np.fliplr(m).T


def IterativeFDKerrCompute(Pic, t_length, s_length, z_length, Size, BetaScanRange, Udomain, Pdomain, Distance, G,
                           t, on_error="raise"):
    """Error slice of the iterative FDK for image slice t (MATLAB index, from 1):
    LBeta * s_length * z_length values laid out [beta][z][s], the derivation of
    the gateway's scalars included (IterativeFDKerrCompute.cpp:5-31).
    BetaScanRange and Udomain are single, Pdomain and G double."""
    pic = _f32(Pic)
    nt, ns, nz = int(t_length), int(s_length), int(z_length)
    if pic.size != nt * ns * nz:
        raise ValueError("Pic must hold t_length*s_length*z_length values")
    Size = _f64(Size)
    beta, U = _f32(BetaScanRange), _f32(Udomain)
    P, G = _f64(Pdomain), _f64(G)
    res = _f64([Size[0] / nt, Size[1] / ns, Size[2] / nz])
    out = np.zeros(len(beta) * ns * nz, np.float32)
    bint = np.float32(abs(beta[1] - beta[0])) if len(beta) > 1 else np.float32(0)
    du = np.float32(abs(U[1] - U[0])) if len(U) > 1 else np.float32(0)
    pint = abs(P[1] - P[0]) if len(P) > 1 else 0.0
    _run("ct_IterativeFDKerrCompute", out, on_error, _ptr(pic), _ptr(out), _ptr(beta), _ptr(U), _ptr(P), _ptr(G),
         _ptr(Size), nt, ns, nz, Size[0] / 2, Size[1] / 2, Size[2] / 2, len(beta), len(P), len(U), len(G),
         float(Distance), _ptr(res), int(t) - 1, float(bint), float(du), float(pint))
    return out.astype(np.float64)


def ImplementUI(R, Xigamadomain, Gamadomain, BetaScanRange, betaStartAngle, MaxGama, Distance, Distance_s2d, Size,
                z_length, on_error="raise"):
    """Curved-detector short-scan FDK (ImplementUI.cpp:5-26): R double
    [beta][xi][gamma] -> float64 column vector of Size[0]*Size[1]*z_length
    values laid out [z][s][t].  Size is cast to int as the gateway does."""
    R = _f64(R)
    xi, gama, beta = _f64(Xigamadomain), _f64(Gamadomain), _f64(BetaScanRange)
    size = np.ascontiguousarray([int(v) for v in np.asarray(Size, np.float64).ravel()[:3]], np.int32)
    nz = int(z_length)
    if R.size != len(xi) * len(gama) * len(beta):
        raise ValueError("R must hold LGama*LXigama*LBeta values")
    out = np.zeros(int(size[0]) * int(size[1]) * nz, np.float64)
    _run("ct_FDKUI", out, on_error, _ptr(out), _ptr(R), _ptr(xi), _ptr(gama), _ptr(beta), float(betaStartAngle),
         float(MaxGama), float(Distance), float(Distance_s2d), len(gama), len(beta), len(xi), _ptr(size), nz)
    return out

